/*
 * kpm_oracle.c — CPU FP64 restatement of the reference's Chebyshev (KPM) path.
 * TEST INFRASTRUCTURE ONLY (checker for tests/, smoke() and bench.py's CPU
 * baseline).  Parity unpinned against the reference's own outputs (it cannot be
 * built here and ships no golden data); pinned by analytic known answers and an
 * independent scipy implementation in tests/.  See kpm_oracle.h.
 *
 * Compiled with -ffp-contract=off so that no multiply-add is fused: the
 * reference's arithmetic is evaluated operation by operation.
 */
#include "kpm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* seeded inputs                                                              */
/* ------------------------------------------------------------------------- */
uint64_t tbo_mix64(uint64_t x) {
  /* SplitMix64 finaliser (Steele, Lea, Flood 2014). */
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

double tbo_u01(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t k = tbo_mix64(seed ^ tbo_mix64(stream + 0x632BE59BD9B4E019ull));
  uint64_t h = tbo_mix64(k + idx * 0xD1B54A32D192ED03ull);
  return (double)(h >> 11) * 0x1.0p-53;
}

void tbo_random_phase_kets(int32_t n, int32_t R, uint64_t seed, double* kets) {
  const double inv = 1.0 / sqrt((double)n);
  const double two_pi = 6.283185307179586476925286766559;
  for (int32_t r = 0; r < R; ++r)
    for (int32_t i = 0; i < n; ++i) {
      double th = two_pi * tbo_u01(seed, (uint64_t)r, (uint64_t)i);
      kets[2 * ((int64_t)r * n + i)] = cos(th) * inv;
      kets[2 * ((int64_t)r * n + i) + 1] = sin(th) * inv;
    }
}

void tbo_uniform_disorder(int32_t n, double W, uint64_t seed, double* v) {
  for (int32_t i = 0; i < n; ++i)
    v[i] = W * (tbo_u01(seed, 0xD150D3Dull, (uint64_t)i) - 0.5);
}

/* ------------------------------------------------------------------------- */
/* n-th nearest-neighbour shells, TB/unit_cell.h:678-707                      */
/* ------------------------------------------------------------------------- */
typedef struct { double d; int32_t to; int32_t v[3]; } nn_item;

static int nn_less(const nn_item* a, const nn_item* b) {
  /* priority: smaller distance first; ties broken by (to, lattice vector)
   * lexicographically — the reference's tie order is implementation-defined
   * (std::priority_queue), the shell *set* is not. */
  if (a->d != b->d) return a->d < b->d;
  if (a->to != b->to) return a->to < b->to;
  for (int k = 0; k < 3; ++k) if (a->v[k] != b->v[k]) return a->v[k] < b->v[k];
  return 0;
}

typedef struct { nn_item* h; int n, cap; } nn_heap;
static void heap_push(nn_heap* q, nn_item it) {
  if (q->n == q->cap) { q->cap = q->cap ? 2 * q->cap : 64; q->h = (nn_item*)realloc(q->h, sizeof(nn_item) * q->cap); }
  int i = q->n++;
  q->h[i] = it;
  while (i > 0) { int p = (i - 1) / 2; if (!nn_less(&q->h[i], &q->h[p])) break; nn_item t = q->h[i]; q->h[i] = q->h[p]; q->h[p] = t; i = p; }
}
static nn_item heap_pop(nn_heap* q) {
  nn_item top = q->h[0];
  q->h[0] = q->h[--q->n];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < q->n && nn_less(&q->h[l], &q->h[m])) m = l;
    if (r < q->n && nn_less(&q->h[r], &q->h[m])) m = r;
    if (m == i) break;
    nn_item t = q->h[i]; q->h[i] = q->h[m]; q->h[m] = t; i = m;
  }
  return top;
}

static double hop_distance(int32_t dim, const double* bases, const double* pos,
                           int32_t from, int32_t to, const int32_t* v) {
  /* displacement_of_hopping: -p_from + bases*v + p_to, TB/unit_cell.h:269-273 */
  double s = 0.0;
  for (int x = 0; x < 3; ++x) {
    double d = 0.0;
    for (int c = 0; c < dim; ++c) d = d + bases[c * 3 + x] * (double)v[c];
    double e = (-pos[from * 3 + x] + d) + pos[to * 3 + x];
    s = s + e * e;
  }
  return sqrt(s);
}

typedef struct { int32_t v[3]; } lv3;
typedef struct { lv3* a; int n, cap; } lvset;
static int lvset_has(const lvset* s, const int32_t* v) {
  for (int i = 0; i < s->n; ++i)
    if (s->a[i].v[0] == v[0] && s->a[i].v[1] == v[1] && s->a[i].v[2] == v[2]) return 1;
  return 0;
}
static void lvset_add(lvset* s, const int32_t* v) {
  if (s->n == s->cap) { s->cap = s->cap ? 2 * s->cap : 64; s->a = (lv3*)realloc(s->a, sizeof(lv3) * s->cap); }
  s->a[s->n].v[0] = v[0]; s->a[s->n].v[1] = v[1]; s->a[s->n].v[2] = v[2]; s->n++;
}

int32_t tbo_nn_shell(int32_t dim, const double* bases, int32_t n_atoms,
                     const double* atom_pos, int32_t from, int32_t nn,
                     int32_t* to_out, int32_t* latv_out, int32_t cap) {
  nn_heap q = {0, 0, 0};
  lvset reg = {0, 0, 0};
  /* NN_vectors: {-1,0,1}^dim minus zero, TB/unit_cell.h:138,666-676 */
  int32_t nnv[26][3]; int n_nnv = 0;
  int lim[3] = {1, dim > 1 ? 1 : 0, dim > 2 ? 1 : 0};
  for (int a = -lim[0]; a <= lim[0]; ++a)
    for (int b = -lim[1]; b <= lim[1]; ++b)
      for (int c = -lim[2]; c <= lim[2]; ++c) {
        if (!a && !b && !c) continue;
        nnv[n_nnv][0] = a; nnv[n_nnv][1] = b; nnv[n_nnv][2] = c; n_nnv++;
      }
  #define ADD_CELL(V) do { if (!lvset_has(&reg, (V))) { lvset_add(&reg, (V)); \
      for (int32_t B = 0; B < n_atoms; ++B) { nn_item it; it.to = B; \
        it.v[0] = (V)[0]; it.v[1] = (V)[1]; it.v[2] = (V)[2]; \
        it.d = hop_distance(dim, bases, atom_pos, from, B, it.v); heap_push(&q, it); } } } while (0)
  int32_t zero[3] = {0, 0, 0};
  ADD_CELL(zero);
  int32_t count = 0;
  for (int32_t shell = 0; shell <= nn; ++shell) {
    nn_item top = q.h[0];
    double d0 = top.d;
    while (fabs(top.d - d0) < 1e-7) {
      for (int k = 0; k < n_nnv; ++k) {
        int32_t w[3] = {top.v[0] + nnv[k][0], top.v[1] + nnv[k][1], top.v[2] + nnv[k][2]};
        ADD_CELL(w);
      }
      heap_pop(&q);
      if (shell == nn) {
        if (count >= cap) { free(q.h); free(reg.a); return -1; }
        to_out[count] = top.to;
        latv_out[3 * count] = top.v[0]; latv_out[3 * count + 1] = top.v[1]; latv_out[3 * count + 2] = top.v[2];
        count++;
      }
      top = q.h[0];
    }
  }
  #undef ADD_CELL
  free(q.h); free(reg.a);
  return count;
}

/* ------------------------------------------------------------------------- */
/* lattice -> triplets -> CSC (Eigen setFromTriplets semantics)               */
/* ------------------------------------------------------------------------- */
int64_t tbo_total_sites(const tbo_lattice* L) {
  int64_t n = L->n_atoms;
  for (int i = 0; i < L->dim; ++i) n *= L->span[i];
  return n;
}

int64_t tbo_compressed_sites(const tbo_lattice* L) {
  int64_t N = tbo_total_sites(L), k = 0;
  if (!L->removed) return N;
  for (int64_t i = 0; i < N; ++i) k += L->removed[i] ? 0 : 1;
  return k;
}

int64_t tbo_triplet_bound(const tbo_lattice* L) {
  return 2 * (tbo_total_sites(L) / L->n_atoms) * (int64_t)L->n_hops;
}

/* span strides: index_bare(i_v, a) = i_v . span_s + a, TB/lattice.h:28,111-114 */
static void span_strides(const tbo_lattice* L, int64_t* s) {
  s[L->dim - 1] = L->n_atoms;
  for (int i = L->dim - 2; i >= 0; --i) s[i] = s[i + 1] * L->span[i + 1];
}

static void atom_position(const tbo_lattice* L, int32_t a, const int32_t* iv, double* r) {
  /* atom_pos[a] + bases * i_v, TB/unit_cell.h:91-92,294-297 */
  for (int x = 0; x < 3; ++x) {
    double d = 0.0;
    for (int c = 0; c < L->dim; ++c) d = d + L->bases[c * 3 + x] * (double)iv[c];
    r[x] = L->atom_pos[a * 3 + x] + d;
  }
}

typedef struct { int32_t row, col; double re, im; } trip;

/* Enumerates cells (row-major, last axis fastest, TB/lattice.h:82-91) x hoppings
 * (table order) and applies the mode's filter, TB/lattice.h:468-483. */
static int64_t make_triplets(const tbo_lattice* L, trip* out, int64_t cap, int32_t* comp_index) {
  const int dim = L->dim;
  int64_t ss[3];
  span_strides(L, ss);
  int64_t n_cells = 1;
  for (int i = 0; i < dim; ++i) n_cells *= L->span[i];
  int64_t k = 0;
  int32_t iv[3] = {0, 0, 0};
  for (int64_t c = 0; c < n_cells; ++c) {
    int64_t rem = c;
    for (int i = dim - 1; i >= 0; --i) { iv[i] = (int32_t)(rem % L->span[i]); rem /= L->span[i]; }
    for (int32_t h = 0; h < L->n_hops; ++h) {
      int32_t from = L->hop_from[h], to = L->hop_to[h];
      int32_t tv[3] = {0, 0, 0}, tvm[3] = {0, 0, 0};
      int inside = 1, ok = 1;
      for (int i = 0; i < dim; ++i) {
        tv[i] = iv[i] + L->hop_latv[3 * h + i];
        int in_i = tv[i] >= 0 && tv[i] < L->span[i];
        inside = inside && in_i;
        if (L->mode == TBO_MODE_PERIODIC_BARE) ok = ok && (L->extend[i] != 0 || in_i);
        /* mod_arr_u: ((x % y) + y) % y with C truncation, TB/lattice.h:222-223 */
        tvm[i] = ((tv[i] % L->span[i]) + L->span[i]) % L->span[i];
      }
      if (L->mode != TBO_MODE_PERIODIC_BARE) ok = inside;
      if (!ok) continue;
      int64_t rb = 0, cb = 0;
      for (int i = 0; i < dim; ++i) {
        rb += iv[i] * ss[i];
        cb += (int64_t)(L->mode == TBO_MODE_PERIODIC_BARE ? tvm[i] : tv[i]) * ss[i];
      }
      rb += from; cb += to;
      int32_t row = (int32_t)rb, col = (int32_t)cb;
      if (L->mode == TBO_MODE_SPARSE && comp_index) {
        if (comp_index[rb] < 0 || comp_index[cb] < 0) continue;   /* TB/lattice.h:270-272 */
        row = comp_index[rb]; col = comp_index[cb];
      }
      double tr = L->hop_t[2 * h], ti = L->hop_t[2 * h + 1];
      if (L->mode != TBO_MODE_BARE) {
        if (L->gauge_kind != TBO_GAUGE_NONE) {
          /* t *= exp(i A(r_from) . d_hop), TB/lattice.h:235-238, 282-285 */
          double A[3], d[3], rf[3];
          int32_t dv[3] = {0, 0, 0};
          for (int i = 0; i < dim; ++i) dv[i] = tv[i] - iv[i];
          if (L->gauge_kind == TBO_GAUGE_LINEAR) {
            atom_position(L, from, iv, rf);
            const double* G = L->gauge_linear;
            for (int x = 0; x < 3; ++x) {
              double s = 0.0;
              for (int y = 0; y < 3; ++y) s = s + G[3 * x + y] * rf[y];
              A[x] = s + G[9 + x];
            }
          } else {
            for (int x = 0; x < 3; ++x) A[x] = L->gauge_site[3 * rb + x];
          }
          for (int x = 0; x < 3; ++x) {
            double dd = 0.0;
            for (int cc = 0; cc < dim; ++cc) dd = dd + L->bases[cc * 3 + x] * (double)dv[cc];
            d[x] = (-L->atom_pos[from * 3 + x] + dd) + L->atom_pos[to * 3 + x];
          }
          double phi = (A[0] * d[0] + A[1] * d[1]) + A[2] * d[2];
          double cr = cos(phi), ci = sin(phi);
          double nr = tr * cr - ti * ci, ni = tr * ci + ti * cr;
          tr = nr; ti = ni;
        }
        if (L->scalar_site && row == col) tr = tr + L->scalar_site[rb];  /* :239, :286 */
      }
      if (k + 2 > cap) return -1;
      if (L->is_complex) {
        out[k].row = row; out[k].col = col; out[k].re = tr; out[k].im = ti; ++k;
        if (row == col) continue;
        out[k].row = col; out[k].col = row; out[k].re = tr; out[k].im = -ti; ++k;
      } else {
        out[k].row = row; out[k].col = col; out[k].re = tr; out[k].im = 0.0; ++k;
        if (row == col) continue;
        out[k].row = col; out[k].col = row; out[k].re = tr; out[k].im = 0.0; ++k;
      }
    }
  }
  return k;
}

/* setFromTriplets: stable counting sort by column, stable insertion sort by row
 * inside each column, duplicates summed left to right (insertion order). */
static int64_t triplets_to_csc(int32_t n, const trip* t, int64_t nt, int32_t is_complex,
                               int32_t* col_ptr, int32_t* row_idx, double* values, int64_t cap) {
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  for (int64_t k = 0; k < nt; ++k) cnt[t[k].col + 1]++;
  for (int32_t j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
  int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
  memcpy(cur, cnt, sizeof(int64_t) * ((size_t)n + 1));
  int64_t* ord = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nt > 0 ? nt : 1));
  for (int64_t k = 0; k < nt; ++k) ord[cur[t[k].col]++] = k;
  int64_t nnz = 0;
  for (int32_t j = 0; j < n; ++j) {
    int64_t b = cnt[j], e = cnt[j + 1];
    for (int64_t p = b + 1; p < e; ++p) {            /* stable insertion sort by row */
      int64_t x = ord[p]; int64_t q = p - 1;
      while (q >= b && t[ord[q]].row > t[x].row) { ord[q + 1] = ord[q]; --q; }
      ord[q + 1] = x;
    }
    col_ptr[j] = (int32_t)nnz;
    for (int64_t p = b; p < e;) {
      int32_t r = t[ord[p]].row;
      double sr = t[ord[p]].re, si = t[ord[p]].im;
      int64_t q = p + 1;
      while (q < e && t[ord[q]].row == r) { sr = sr + t[ord[q]].re; si = si + t[ord[q]].im; ++q; }
      if (nnz >= cap) { free(cnt); free(cur); free(ord); return -1; }
      row_idx[nnz] = r;
      if (is_complex) { values[2 * nnz] = sr; values[2 * nnz + 1] = si; }
      else values[nnz] = sr;
      ++nnz;
      p = q;
    }
  }
  col_ptr[n] = (int32_t)nnz;
  free(cnt); free(cur); free(ord);
  return nnz;
}

int64_t tbo_build_csc(const tbo_lattice* L, int32_t* col_ptr, int32_t* row_idx,
                      double* values, int64_t cap) {
  int64_t N = tbo_total_sites(L);
  int32_t* comp = NULL;
  int32_t n_rows = (int32_t)N;
  if (L->mode == TBO_MODE_SPARSE && L->removed) {
    comp = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);   /* index_comp_construct :447-457 */
    int32_t c = 0;
    for (int64_t i = 0; i < N; ++i) comp[i] = L->removed[i] ? -1 : c++;
    /* Note: the reference sizes the matrix total_number x total_number even with
     * vacancies (TB/lattice.h:300); trailing rows/columns stay empty. */
  }
  int64_t bound = tbo_triplet_bound(L);
  trip* t = (trip*)malloc(sizeof(trip) * (size_t)(bound > 0 ? bound : 1));
  int64_t nt = make_triplets(L, t, bound, comp);
  int64_t nnz = nt < 0 ? -1 : triplets_to_csc(n_rows, t, nt, L->is_complex, col_ptr, row_idx, values, cap);
  free(t); free(comp);
  return nnz;
}

int64_t tbo_position_diag(const tbo_lattice* L, int32_t axis, double* x_out) {
  /* op_position, TB/lattice.h:313-336: index_sequence (cells row-major) x atoms. */
  if (axis >= L->dim) axis = 0;
  int64_t N = tbo_total_sites(L), n_cells = N / L->n_atoms, k = 0;
  int32_t iv[3] = {0, 0, 0};
  for (int64_t c = 0; c < n_cells; ++c) {
    int64_t rem = c;
    for (int i = L->dim - 1; i >= 0; --i) { iv[i] = (int32_t)(rem % L->span[i]); rem /= L->span[i]; }
    for (int32_t a = 0; a < L->n_atoms; ++a) {
      int64_t b = c * L->n_atoms + a;
      if (L->removed && L->removed[b]) continue;
      double d = 0.0;
      for (int cc = 0; cc < L->dim; ++cc) d = d + L->bases[cc * 3 + axis] * (double)iv[cc];
      x_out[k++] = L->atom_pos[a * 3 + axis] + d;
    }
  }
  return k;
}

/* ------------------------------------------------------------------------- */
/* rescale (H - b I)/a: sparse difference with the identity (pattern union)   */
/* ------------------------------------------------------------------------- */
int64_t tbo_rescale_csc(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                        int32_t cplx, double a, double b, int32_t* ocp, int32_t* ori,
                        double* ov, int64_t cap) {
  int64_t k = 0;
  for (int32_t j = 0; j < n; ++j) {
    ocp[j] = (int32_t)k;
    int diag_done = 0;
    for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
      int32_t r = ri[p];
      if (!diag_done && r > j) {                    /* identity-only entry: (0 - b)/a */
        if (k >= cap) return -1;
        ori[k] = j;
        if (cplx) { ov[2 * k] = (0.0 - b) / a; ov[2 * k + 1] = (0.0 - 0.0) / a; } else ov[k] = (0.0 - b) / a;
        ++k; diag_done = 1;
      }
      if (k >= cap) return -1;
      ori[k] = r;
      if (r == j) {                                   /* both: (h - b)/a */
        if (cplx) { ov[2 * k] = (v[2 * p] - b) / a; ov[2 * k + 1] = (v[2 * p + 1] - 0.0) / a; }
        else ov[k] = (v[p] - b) / a;
        diag_done = 1;
      } else {                                        /* H only: (h - 0)/a */
        if (cplx) { ov[2 * k] = (v[2 * p] - 0.0) / a; ov[2 * k + 1] = (v[2 * p + 1] - 0.0) / a; }
        else ov[k] = (v[p] - 0.0) / a;
      }
      ++k;
    }
    if (!diag_done) {
      if (k >= cap) return -1;
      ori[k] = j;
      if (cplx) { ov[2 * k] = (0.0 - b) / a; ov[2 * k + 1] = (0.0 - 0.0) / a; } else ov[k] = (0.0 - b) / a;
      ++k;
    }
  }
  ocp[n] = (int32_t)k;
  return k;
}

void tbo_commutator_values(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                           int32_t cplx, const double* x, double* ov) {
  for (int32_t j = 0; j < n; ++j)
    for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
      int32_t i = ri[p];
      if (cplx) {
        ov[2 * p] = x[i] * v[2 * p] - v[2 * p] * x[j];
        ov[2 * p + 1] = x[i] * v[2 * p + 1] - v[2 * p + 1] * x[j];
      } else {
        ov[p] = x[i] * v[p] - v[p] * x[j];
      }
    }
}

/* ------------------------------------------------------------------------- */
/* sparse (CSC) x dense column-major complex                                  */
/* ------------------------------------------------------------------------- */
static void csc_mult_col(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                         int32_t cplx, const double* x, double* y) {
  memset(y, 0, sizeof(double) * 2 * (size_t)n);
  for (int32_t j = 0; j < n; ++j) {
    double xr = x[2 * j], xi = x[2 * j + 1];
    for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
      int32_t i = ri[p];
      if (cplx) {
        double hr = v[2 * p], hi = v[2 * p + 1];
        y[2 * i] += hr * xr - hi * xi;
        y[2 * i + 1] += hr * xi + hi * xr;
      } else {
        y[2 * i] += v[p] * xr;
        y[2 * i + 1] += v[p] * xi;
      }
    }
  }
}

void tbo_csc_mult(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                  int32_t cplx, int32_t R, const double* x, double* y) {
  for (int32_t r = 0; r < R; ++r)
    csc_mult_col(n, cp, ri, v, cplx, x + 2 * (int64_t)r * n, y + 2 * (int64_t)r * n);
}

double tbo_trace_braket(int32_t n, int32_t R, const double* A, const double* B) {
  /* loop order of TB/numerical.h:129-133: rows outer, columns inner */
  double t = 0.0;
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = 0; j < R; ++j) {
      int64_t q = 2 * ((int64_t)j * n + i);
      t += A[q] * B[q] + A[q + 1] * B[q + 1];
    }
  return t;
}

void tbo_trace_braket_complex(int32_t n, int32_t R, const double* A, const double* B, double* o) {
  double sr = 0.0, si = 0.0;
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = 0; j < R; ++j) {
      int64_t q = 2 * ((int64_t)j * n + i);
      /* conj(a) * b */
      sr += A[q] * B[q] + A[q + 1] * B[q + 1];
      si += A[q] * B[q + 1] - A[q + 1] * B[q];
    }
  o[0] = sr; o[1] = si;
}

/* per-column Re <b|t>, summed over the column */
static double col_braket(int32_t n, const double* b, const double* t) {
  double s = 0.0;
  for (int32_t i = 0; i < n; ++i) s += b[2 * i] * t[2 * i] + b[2 * i + 1] * t[2 * i + 1];
  return s;
}

int32_t tbo_cheb_moments(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                         int32_t cplx, int32_t n_mom, const double* bras, const double* kets,
                         int32_t R, double* mu, int32_t threads, int32_t steps_limit) {
  if (n_mom < 2 || R < 1 || n < 1) return -1;
  int32_t last = n_mom;                       /* moments 0 .. last-1 */
  if (steps_limit > 0 && steps_limit + 1 < n_mom) last = steps_limit + 1;
  double* part = (double*)calloc((size_t)R * (size_t)n_mom, sizeof(double));
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
  for (int32_t r = 0; r < R; ++r) {
    /* Tn_2 = kets, Tn_1 = M kets, Tn = 2 M Tn_1 - Tn_2 (TB/numerical.h:367-377),
     * one column at a time (Eigen's product is column by column as well). */
    double* a = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    double* b = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    double* c = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    const double* br = bras + 2 * (int64_t)r * n;
    memcpy(a, kets + 2 * (int64_t)r * n, sizeof(double) * 2 * (size_t)n);
    csc_mult_col(n, cp, ri, v, cplx, a, b);
    part[(int64_t)r * n_mom + 0] = col_braket(n, br, a);
    part[(int64_t)r * n_mom + 1] = col_braket(n, br, b);
    for (int32_t k = 2; k < last; ++k) {
      csc_mult_col(n, cp, ri, v, cplx, b, c);
      for (int32_t i = 0; i < 2 * n; ++i) c[i] = 2.0 * c[i] - a[i];
      part[(int64_t)r * n_mom + k] = col_braket(n, br, c);
      double* t = a; a = b; b = c; c = t;
    }
    free(a); free(b); free(c);
  }
  (void)threads;
  for (int32_t k = 0; k < n_mom; ++k) {
    double s = 0.0;
    for (int32_t r = 0; r < R; ++r) s += part[(int64_t)r * n_mom + k];
    mu[k] = k < last ? s : 0.0;
  }
  free(part);
  return 0;
}

int32_t tbo_cheb_blocks(int32_t n, const int32_t* cp, const int32_t* ri, const double* v,
                        int32_t cplx, int32_t n_mom, const double* x0, int32_t R, double* out) {
  if (n_mom < 1) return -1;
  int64_t blk = 2 * (int64_t)n * R;
  memcpy(out, x0, sizeof(double) * (size_t)blk);
  if (n_mom == 1) return 0;
  tbo_csc_mult(n, cp, ri, v, cplx, R, out, out + blk);
  for (int32_t k = 2; k < n_mom; ++k) {
    double* y = out + k * blk;
    tbo_csc_mult(n, cp, ri, v, cplx, R, out + (k - 1) * blk, y);
    const double* z = out + (k - 2) * blk;
    for (int64_t i = 0; i < blk; ++i) y[i] = 2.0 * y[i] - z[i];
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* kernels, TB/numerical.h:393-447                                            */
/* ------------------------------------------------------------------------- */
void tbo_kernel_seq(int32_t kind, int32_t N, double p0, double p1, double* g) {
  const double pi = 3.14159265358979323846;
  for (int32_t n = 0; n < N; ++n) {
    double x = 1.0;
    switch (kind) {
      case TBO_K_DIRICHLET: x = 1.0; break;
      case TBO_K_FEJER: x = 1.0 - (double)n / N; break;
      case TBO_K_LORENTZ: x = sinh(p0 * (1.0 - (double)n / N)) / sinh(p0); break;
      case TBO_K_JACKSON: {
        int32_t N1 = N + 1;
        double s1 = pi / N1, s2 = n * s1;
        x = ((N1 - n) * cos(s2) + sin(s2) / tan(s1)) / N1;
        break;
      }
      case TBO_K_LANCZOS: {
        double piN = pi / N;
        x = pow(sin(n * piN) / piN, p0);  /* as written in the reference (n=0 gives 0) */
        break;
      }
      case TBO_K_WANG_ZUNGER: x = exp(-pow(n * (p0 / N), p1)); break;
    }
    g[n] = x;
  }
}

/* ------------------------------------------------------------------------- */
/* reconstruction                                                             */
/* ------------------------------------------------------------------------- */
static void csqrt_(double re, double im, double* o) {
  /* principal square root (std::sqrt(complex)) */
  double m = hypot(re, im);
  double sr = sqrt(0.5 * (m + fabs(re)));
  if (sr == 0.0) { o[0] = 0.0; o[1] = 0.0; return; }
  if (re >= 0.0) { o[0] = sr; o[1] = im / (2.0 * sr); }
  else { o[0] = fabs(im) / (2.0 * sr); o[1] = im < 0.0 || (im == 0.0 && signbit(im)) ? -sr : sr; }
}
static void cmul_(const double* a, const double* b, double* o) {
  double r = a[0] * b[0] - a[1] * b[1], i = a[0] * b[1] + a[1] * b[0];
  o[0] = r; o[1] = i;
}
static void cdiv_(const double* a, const double* b, double* o) {
  double d = b[0] * b[0] + b[1] * b[1];
  double r = (a[0] * b[0] + a[1] * b[1]) / d, i = (a[1] * b[0] - a[0] * b[1]) / d;
  o[0] = r; o[1] = i;
}

void tbo_expn_coef_alpha_seq(double zr, double zi, int32_t n, double* out) {
  /* s1 = sqrt(1 - z^2); s2 = z - i s1; sn = -2i/s1; g0 = -i/s1; g_k = sn * s2^k */
  double z[2] = {zr, zi}, zz[2], s1[2], s2[2], sn[2];
  cmul_(z, z, zz);
  double om[2] = {1.0 - zz[0], 0.0 - zz[1]};
  csqrt_(om[0], om[1], s1);
  s2[0] = z[0] + s1[1]; s2[1] = z[1] - s1[0];          /* z - i*s1 */
  double m2i[2] = {0.0, -2.0}, mi[2] = {0.0, -1.0};
  cdiv_(m2i, s1, sn);
  if (n > 0) cdiv_(mi, s1, out);
  for (int32_t k = 1; k < n; ++k) {
    double t[2];
    cmul_(sn, s2, t); sn[0] = t[0]; sn[1] = t[1];
    out[2 * k] = sn[0]; out[2 * k + 1] = sn[1];
  }
}

double tbo_green_imag_eval(int32_t n, const double* g, const double* mu, double zr, double zi) {
  double* al = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  tbo_expn_coef_alpha_seq(zr, zi, n, al);
  double s = 0.0;
  for (int32_t k = 0; k < n; ++k) s += g[k] * al[2 * k + 1] * mu[k];
  free(al);
  return s;
}

void tbo_green_imag_fft(int32_t n, const double* g, const double* mu, int32_t up,
                        double* E, double* val) {
  const double pi = 3.14159265358979323846;
  int32_t N = n * (up > 0 ? up : 1);
  for (int32_t k = 0; k < N; ++k) {
    double th = 0.5 * pi / N + k * (pi / N);           /* utils::range(0.5pi/N, pi/N, N) */
    double y = g[0] * mu[0];
    for (int32_t m = 1; m < n; ++m) y += 2.0 * (g[m] * mu[m]) * cos(pi * m * (k + 0.5) / N);
    E[k] = cos(th);
    val[k] = y * (1.0 / sqrt(1.0 - E[k] * E[k]));
  }
}

/* ------------------------------------------------------------------------- */
/* Kubo                                                                       */
/* ------------------------------------------------------------------------- */
void tbo_mu_nm(int32_t M, int64_t K, const double* L, const double* Rb, double* out) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int32_t m = 0; m < M; ++m)
    for (int32_t n = 0; n < M; ++n) {
      const double* a = L + 2 * (int64_t)m * K;
      const double* b = Rb + 2 * (int64_t)n * K;
      double sr = 0.0, si = 0.0;
      for (int64_t k = 0; k < K; ++k) {
        sr += a[2 * k] * b[2 * k] + a[2 * k + 1] * b[2 * k + 1];
        si += a[2 * k] * b[2 * k + 1] - a[2 * k + 1] * b[2 * k];
      }
      out[2 * ((int64_t)m * M + n)] = sr;
      out[2 * ((int64_t)m * M + n) + 1] = si;
    }
}

void tbo_bastin_zeta(int32_t M, const double* mu, int32_t n_eps, const double* eps,
                     double vol, double* zeta) {
  for (int32_t e = 0; e < n_eps; ++e) {
    double x = eps[e], s = sqrt(1.0 - x * x), th = acos(x);
    double zr = 0.0, zi = 0.0;
    for (int32_t m = 0; m < M; ++m) {
      double am = m == 0 ? 1.0 : 2.0, Tm = cos(m * th);
      for (int32_t n = 0; n < M; ++n) {
        double an = n == 0 ? 1.0 : 2.0, Tn = cos(n * th);
        /* Gamma = a_m a_n [(x - i n s) e^{i n th} T_m + (x + i m s) e^{-i m th} T_n] */
        double c1 = cos(n * th), s1 = sin(n * th), c2 = cos(m * th), s2 = -sin(m * th);
        double g1r = x * c1 + n * s * s1, g1i = x * s1 - n * s * c1;      /* (x - i n s)(c1 + i s1) */
        double g2r = x * c2 - m * s * s2, g2i = x * s2 + m * s * c2;      /* (x + i m s)(c2 + i s2) */
        double Gr = am * an * (g1r * Tm + g2r * Tn), Gi = am * an * (g1i * Tm + g2i * Tn);
        double ur = mu[2 * ((int64_t)m * M + n)], ui = mu[2 * ((int64_t)m * M + n) + 1];
        zr += ur * Gr - ui * Gi;
        zi += ur * Gi + ui * Gr;
      }
    }
    double den = (1.0 - x * x) * (1.0 - x * x) * vol;
    zeta[2 * e] = zr / den;
    zeta[2 * e + 1] = zi / den;
  }
}

void tbo_greenwood_sigma(int32_t M, const double* mu, int32_t n_eps, const double* eps,
                         double R, double* sigma) {
  for (int32_t e = 0; e < n_eps; ++e) {
    double x = eps[e], th = acos(x), sr = 0.0;
    for (int32_t m = 0; m < M; ++m) {
      double am = m == 0 ? 1.0 : 2.0, Tm = cos(m * th);
      for (int32_t n = 0; n < M; ++n) {
        double an = n == 0 ? 1.0 : 2.0, Tn = cos(n * th);
        sr += mu[2 * ((int64_t)m * M + n)] * am * an * Tm * Tn;
      }
    }
    sigma[e] = -sr / (1.0 - x * x) / R;
  }
}

/* Bastin integration, TB/snippets.h:421-449: drop N/24 nodes at each end,
 * reverse to ascending energy, cumulative trapezoid from the first node above 0
 * with the half-cell weights there.  zeta: N complex (interleaved). Returns n. */
int32_t tbo_bastin_integrate(int32_t N, const double* eps, const double* zeta, double* E, double* re, double* im) {
  int32_t cut = N / 24, n = N - 2 * cut;
  double* zr = (double*)malloc(sizeof(double) * (size_t)n);
  double* zi = (double*)malloc(sizeof(double) * (size_t)n);
  for (int32_t k = 0; k < n; ++k) {
    int32_t s = cut + (n - 1 - k);
    E[k] = eps[s]; zr[k] = zeta[2 * s]; zi[k] = zeta[2 * s + 1];
    re[k] = 0.0; im[k] = 0.0;
  }
  int32_t e0 = 0;
  while (e0 < n && !(E[e0] > 0.0)) ++e0;       /* upper_bound(E, 0.0) */
  re[e0] = (zr[e0] * 3 / 4 + zr[e0 - 1] / 4) * (E[e0] - E[e0 - 1]) / 2;
  re[e0 - 1] = -(zr[e0] / 4 + zr[e0 - 1] * 3 / 4) * (E[e0] - E[e0 - 1]) / 2;
  for (int32_t i = e0 + 1; i < n; ++i) {
    re[i] = re[i - 1] + (zr[i] + zr[i - 1]) / 2 * (E[i] - E[i - 1]);
    im[i] = im[i - 1] + (zi[i] + zi[i - 1]) / 2 * (E[i] - E[i - 1]);
  }
  for (int32_t i = e0 - 2; i >= 0; --i) {
    re[i] = re[i + 1] - (zr[i] + zr[i + 1]) / 2 * (E[i + 1] - E[i]);
    im[i] = im[i + 1] - (zi[i] + zi[i + 1]) / 2 * (E[i + 1] - E[i]);
  }
  free(zr); free(zi);
  return n;
}
