// host_model.cpp — unit cell, n-th nearest-neighbour shells and lattice spec
// (host side of the builder).  Restates the reference's host model:
//   UnitCell ctor / add_hopping / add_hopping_direct  TB/unit_cell.h:188-256, 527-547
//   UnitCellNN::generate_hoppings_to / add_cell      TB/unit_cell.h:678-707
//   PartialLattice ctor / set_scalar_field            TB/lattice.h:105-117, 495-505
// The hopping table is kept in insertion order, which is the enumeration order
// the device builder uses (the reference iterates an unordered_map, whose order
// is implementation-defined; the resulting CSC structure does not depend on it).
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <map>
#include <queue>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "host_model.h"

namespace tbk {

static thread_local std::string g_last_error;
static thread_local int g_last_code = 0;
thread_local const AsyncAllocCtx* tl_async_alloc = nullptr;

void set_error(int code, const std::string& msg) { g_last_code = code; g_last_error = msg; }

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_error(code, buf);
  return code;
}

double Cell::hop_distance(int from, int to, const int32_t* v) const {
  double s = 0.0;
  for (int x = 0; x < 3; ++x) {
    double d = 0.0;
    for (int c = 0; c < dim; ++c) d = d + bases[c * 3 + x] * (double)v[c];
    double e = (-pos[from * 3 + x] + d) + pos[to * 3 + x];
    s = s + e * e;
  }
  return std::sqrt(s);
}

int Cell::find_hop(int from, int to, const int32_t* v) const {
  for (size_t k = 0; k < hops.size(); ++k) {
    const Hop& h = hops[k];
    if (h.from == from && h.to == to && h.v[0] == v[0] && h.v[1] == v[1] && h.v[2] == v[2])
      return (int)k;
  }
  return -1;
}

bool Cell::hopping_exists(int from, int to, const int32_t* v) const {
  int32_t w[3] = {-v[0], -v[1], -v[2]};
  return find_hop(from, to, v) >= 0 || find_hop(to, from, w) >= 0;
}

void Cell::add_direct(int from, int to, const int32_t* v, double tr, double ti) {
  if (hopping_exists(from, to, v)) { ++warnings; return; }              // "Hopping already exists"
  bool onsite = from == to && v[0] == 0 && v[1] == 0 && v[2] == 0;
  if (onsite && ti != 0.0) { ++warnings; return; }                     // "On-site hopping must be real"
  Hop h;
  if (from < to) {                                                      // store h.c. so that from >= to
    h.from = to; h.to = from; h.v[0] = -v[0]; h.v[1] = -v[1]; h.v[2] = -v[2]; h.tr = tr; h.ti = -ti;
  } else {
    h.from = from; h.to = to; h.v[0] = v[0]; h.v[1] = v[1]; h.v[2] = v[2]; h.tr = tr; h.ti = ti;
  }
  hops.push_back(h);
}

namespace {
struct NNItem {
  double d;
  int to;
  int32_t v[3];
};
struct NNGreater {  // min-heap on distance; ties by (to, lattice vector)
  bool operator()(const NNItem& a, const NNItem& b) const {
    if (a.d != b.d) return a.d > b.d;
    if (a.to != b.to) return a.to > b.to;
    for (int k = 0; k < 3; ++k) if (a.v[k] != b.v[k]) return a.v[k] > b.v[k];
    return false;
  }
};
}  // namespace

int Cell::nn_shell(int from, int nn, std::vector<std::array<int32_t, 4>>& out) const {
  std::priority_queue<NNItem, std::vector<NNItem>, NNGreater> q;
  std::set<std::array<int32_t, 3>> reg;
  std::vector<std::array<int32_t, 3>> nnv;
  int lim1 = dim > 1 ? 1 : 0, lim2 = dim > 2 ? 1 : 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -lim1; b <= lim1; ++b)
      for (int c = -lim2; c <= lim2; ++c)
        if (a || b || c) nnv.push_back({a, b, c});
  auto add_cell = [&](const std::array<int32_t, 3>& v) {
    if (reg.count(v)) return;
    reg.insert(v);
    for (int B = 0; B < n_atoms; ++B) {
      NNItem it;
      it.to = B; it.v[0] = v[0]; it.v[1] = v[1]; it.v[2] = v[2];
      it.d = hop_distance(from, B, it.v);
      q.push(it);
    }
  };
  add_cell({0, 0, 0});
  out.clear();
  for (int shell = 0; shell <= nn; ++shell) {
    NNItem top = q.top();
    double d0 = top.d;
    while (std::fabs(top.d - d0) < 1e-7) {
      for (auto& dv : nnv) add_cell({top.v[0] + dv[0], top.v[1] + dv[1], top.v[2] + dv[2]});
      q.pop();
      if (shell == nn) out.push_back({top.to, top.v[0], top.v[1], top.v[2]});
      top = q.top();
    }
  }
  return 0;
}

}  // namespace tbk

using tbk::fail;

extern "C" {

const char* tbk_last_error(void) { return tbk::g_last_error.c_str(); }
int tbk_version(void) { return 10000; }

int tbk_cell_create(tbk_cell* out, int32_t dim, const double* lv, int32_t n_atoms,
                    const char* const* names, const double* positions) {
  if (!out || !lv || !positions || !names) return fail(TBK_ERR_INVALID, "tbk_cell_create: null argument");
  *out = nullptr;
  if (dim < 1 || dim > 3) return fail(TBK_ERR_INVALID, "Number of lattice vectors must be equal to the dimension of the unit cell");
  if (n_atoms < 1) return fail(TBK_ERR_INVALID, "Unit cell must contain at least one atom");
  auto* c = new tbk_cell_s();
  c->dim = dim;
  c->n_atoms = n_atoms;
  for (int i = 0; i < 9; ++i) c->bases[i] = 0.0;
  for (int v = 0; v < dim; ++v) {
    bool zero = lv[3 * v] == 0.0 && lv[3 * v + 1] == 0.0 && lv[3 * v + 2] == 0.0;
    if (zero) { delete c; return fail(TBK_ERR_INVALID, "Lattice vectors must not be zero"); }
    for (int x = 0; x < 3; ++x) c->bases[v * 3 + x] = lv[3 * v + x];
  }
  for (int a = 0; a < n_atoms; ++a) {
    std::string nm = names[a] ? names[a] : "";
    for (auto& e : c->names)
      if (e == nm) { delete c; return fail(TBK_ERR_INVALID, "Atom %s is already defined", nm.c_str()); }
    c->names.push_back(nm);
    for (int x = 0; x < 3; ++x) c->pos.push_back(positions[3 * a + x]);
  }
  *out = c;
  return TBK_OK;
}

int tbk_cell_copy(tbk_cell* out, tbk_cell src) {
  if (!out || !src) return fail(TBK_ERR_INVALID, "tbk_cell_copy: null argument");
  *out = new tbk_cell_s(*src);
  return TBK_OK;
}

void tbk_cell_destroy(tbk_cell cell) { delete cell; }

int tbk_cell_atom_index(tbk_cell c, const char* name, int32_t* index) {
  if (!c || !name || !index) return fail(TBK_ERR_INVALID, "tbk_cell_atom_index: null argument");
  for (size_t a = 0; a < c->names.size(); ++a)
    if (c->names[a] == name) { *index = (int32_t)a; return TBK_OK; }
  return fail(TBK_ERR_INVALID, "Atom %s not found in the unit cell", name);
}

int tbk_cell_add_hopping(tbk_cell c, const char* from, const char* to, const int32_t* v,
                         double tr, double ti) {
  if (!c || !from || !to || !v) return fail(TBK_ERR_INVALID, "tbk_cell_add_hopping: null argument");
  c->warnings = 0;
  int32_t f, t;
  TBK_TRY(tbk_cell_atom_index(c, from, &f));
  TBK_TRY(tbk_cell_atom_index(c, to, &t));
  int32_t w[3] = {0, 0, 0};
  for (int i = 0; i < c->dim; ++i) w[i] = v[i];
  if (f == t && w[0] == 0 && w[1] == 0 && w[2] == 0 && ti != 0.0) { c->warnings = 1; return TBK_OK; }
  c->add_direct(f, t, w, tr, ti);
  return TBK_OK;
}

int tbk_cell_add_hopping_nn(tbk_cell c, const char* from, int32_t nn, double tr, double ti) {
  if (!c || !from) return fail(TBK_ERR_INVALID, "tbk_cell_add_hopping_nn: null argument");
  if (nn < 0) return fail(TBK_ERR_INVALID, "neighbour order must be >= 0");
  c->warnings = 0;
  int32_t f;
  TBK_TRY(tbk_cell_atom_index(c, from, &f));
  if (nn == 0) {                               // On_Site
    if (ti != 0.0) { c->warnings = 1; return TBK_OK; }
    int32_t z[3] = {0, 0, 0};
    c->add_direct(f, f, z, tr, ti);
    return TBK_OK;
  }
  std::vector<std::array<int32_t, 4>> shell;
  c->nn_shell(f, nn, shell);
  for (auto& s : shell) {
    int32_t w[3] = {s[1], s[2], s[3]};
    c->add_direct(f, s[0], w, tr, ti);
  }
  return TBK_OK;
}

int tbk_cell_info(tbk_cell c, int32_t* dim, int32_t* n_atoms, int32_t* n_hops) {
  if (!c) return fail(TBK_ERR_INVALID, "tbk_cell_info: null cell");
  if (dim) *dim = c->dim;
  if (n_atoms) *n_atoms = c->n_atoms;
  if (n_hops) *n_hops = (int32_t)c->hops.size();
  return TBK_OK;
}

int tbk_cell_get_hoppings(tbk_cell c, int32_t* from, int32_t* to, int32_t* latv3, double* t2) {
  if (!c) return fail(TBK_ERR_INVALID, "tbk_cell_get_hoppings: null cell");
  for (size_t k = 0; k < c->hops.size(); ++k) {
    const auto& h = c->hops[k];
    if (from) from[k] = h.from;
    if (to) to[k] = h.to;
    if (latv3) for (int i = 0; i < 3; ++i) latv3[3 * k + i] = h.v[i];
    if (t2) { t2[2 * k] = h.tr; t2[2 * k + 1] = h.ti; }
  }
  return TBK_OK;
}

int tbk_cell_get_geometry(tbk_cell c, double* bases, double* positions) {
  if (!c) return fail(TBK_ERR_INVALID, "tbk_cell_get_geometry: null cell");
  if (bases) for (int i = 0; i < 3 * c->dim; ++i) bases[i] = c->bases[i];
  if (positions) for (size_t i = 0; i < c->pos.size(); ++i) positions[i] = c->pos[i];
  return TBK_OK;
}

int tbk_cell_last_warnings(tbk_cell c, int32_t* count) {
  if (!c || !count) return fail(TBK_ERR_INVALID, "tbk_cell_last_warnings: null argument");
  *count = c->warnings;
  return TBK_OK;
}

// ---------------------------------------------------------------- lattice
int tbk_lattice_create(tbk_lattice* out, tbk_cell cell, const int32_t* span) {
  if (!out || !cell || !span) return fail(TBK_ERR_INVALID, "tbk_lattice_create: null argument");
  *out = nullptr;
  int64_t n = cell->n_atoms;
  for (int i = 0; i < cell->dim; ++i) {
    if (span[i] < 1) return fail(TBK_ERR_INVALID, "span must be >= 1 on every axis");
    n *= span[i];
  }
  if (n > INT32_MAX) return fail(TBK_ERR_UNSUPPORTED, "lattice of %lld sites exceeds int32 indexing", (long long)n);
  auto* L = new tbk_lattice_s();
  L->cell = *cell;
  L->span[0] = L->span[1] = L->span[2] = 1;
  for (int i = 0; i < cell->dim; ++i) L->span[i] = span[i];
  L->total = n;
  *out = L;
  return TBK_OK;
}

void tbk_lattice_destroy(tbk_lattice lat) { delete lat; }

int tbk_lattice_total_number(tbk_lattice L, int64_t* n) {
  if (!L || !n) return fail(TBK_ERR_INVALID, "tbk_lattice_total_number: null argument");
  *n = L->total;
  return TBK_OK;
}

int tbk_lattice_set_gauge_linear(tbk_lattice L, const double* G, const double* c) {
  if (!L || !G || !c) return fail(TBK_ERR_INVALID, "tbk_lattice_set_gauge_linear: null argument");
  L->gauge_kind = tbk::GAUGE_LINEAR;
  for (int i = 0; i < 9; ++i) L->gauge_linear[i] = G[i];
  for (int i = 0; i < 3; ++i) L->gauge_linear[9 + i] = c[i];
  L->gauge_sites.clear();
  return TBK_OK;
}

int tbk_lattice_set_gauge_sites(tbk_lattice L, const double* A) {
  if (!L || !A) return fail(TBK_ERR_INVALID, "tbk_lattice_set_gauge_sites: null argument");
  L->gauge_kind = tbk::GAUGE_SITES;
  L->gauge_sites.assign(A, A + 3 * L->total);
  return TBK_OK;
}

int tbk_lattice_clear_gauge(tbk_lattice L) {
  if (!L) return fail(TBK_ERR_INVALID, "tbk_lattice_clear_gauge: null lattice");
  L->gauge_kind = tbk::GAUGE_NONE;
  L->gauge_sites.clear();
  return TBK_OK;
}

static void add_onsite_zeros(tbk::Cell& c) {
  // set_scalar_field adds a zero on-site hopping to every atom that has none,
  // TB/lattice.h:499-504
  for (int i = 0; i < c.n_atoms; ++i) {
    int32_t z[3] = {0, 0, 0};
    if (c.hopping_exists(i, i, z)) continue;
    c.add_direct(i, i, z, 0.0, 0.0);
  }
}

int tbk_lattice_set_scalar_sites(tbk_lattice L, const double* V) {
  if (!L || !V) return fail(TBK_ERR_INVALID, "tbk_lattice_set_scalar_sites: null argument");
  L->scalar_kind = tbk::SCALAR_SITES;
  L->scalar_sites.assign(V, V + L->total);
  add_onsite_zeros(L->cell);
  return TBK_OK;
}

int tbk_lattice_set_scalar_disorder(tbk_lattice L, double W, uint64_t seed) {
  if (!L) return fail(TBK_ERR_INVALID, "tbk_lattice_set_scalar_disorder: null lattice");
  L->scalar_kind = tbk::SCALAR_DISORDER;
  L->disorder_W = W;
  L->disorder_seed = seed;
  L->scalar_sites.clear();
  add_onsite_zeros(L->cell);
  return TBK_OK;
}

int tbk_lattice_set_removed(tbk_lattice L, const uint8_t* removed) {
  if (!L) return fail(TBK_ERR_INVALID, "tbk_lattice_set_removed: null lattice");
  if (!removed) { L->removed.clear(); return TBK_OK; }
  L->removed.assign(removed, removed + L->total);
  return TBK_OK;
}

static int lattice_atom(tbk_lattice L, const char* atom, const char* fn, int* a) {
  if (!L || !atom) return fail(TBK_ERR_INVALID, "%s: null argument", fn);
  for (size_t i = 0; i < L->cell.names.size(); ++i)
    if (L->cell.names[i] == atom) { *a = (int)i; return TBK_OK; }
  return fail(TBK_ERR_INVALID, "Atom %s does not exist in the unit cell.", atom);
}

int tbk_lattice_remove_atoms(tbk_lattice L, const char* atom, const int32_t* cells, int64_t n) {
  int a = 0;
  TBK_TRY(lattice_atom(L, atom, "tbk_lattice_remove_atoms", &a));
  if (n < 0 || (n > 0 && !cells)) return fail(TBK_ERR_INVALID, "tbk_lattice_remove_atoms: bad cell list");
  const int dim = L->cell.dim, na = L->cell.n_atoms;
  std::vector<int64_t> idx((size_t)n);
  for (int64_t k = 0; k < n; ++k) {
    // index_bare(i_v, a) = i_v . span_s + a (row-major cells, atom fastest)
    int64_t c = 0;
    for (int i = 0; i < dim; ++i) {
      const int32_t v = cells[k * dim + i];
      if (v < 0 || v >= L->span[i])
        return fail(TBK_ERR_INVALID, "tbk_lattice_remove_atoms: cell %lld outside the lattice", (long long)k);
      c = c * L->span[i] + v;
    }
    idx[(size_t)k] = c * na + a;
  }
  if (L->removed.empty()) L->removed.assign((size_t)L->total, 0);
  for (int64_t b : idx) L->removed[(size_t)b] = 1;
  return TBK_OK;
}

int tbk_lattice_remove_atoms_random(tbk_lattice L, const char* atom, int64_t n, uint64_t seed) {
  int a = 0;
  TBK_TRY(lattice_atom(L, atom, "tbk_lattice_remove_atoms_random", &a));
  const int64_t cells = L->total / L->cell.n_atoms;
  if (n < 0 || n > cells) return fail(TBK_ERR_INVALID, "The random selection is larger than the total number.");
  // n distinct cells out of `cells`, seeded: Floyd's sampling (Bentley & Floyd,
  // CACM 30(9), 1987) -- for j = cells-n .. cells-1 draw t in [0, j]; take t,
  // or j when t is already taken.  The draws are the counter-based u01 stream.
  std::set<int64_t> pick;
  for (int64_t j = cells - n; j < cells; ++j) {
    int64_t t = (int64_t)(tbk::u01(seed, tbk::kRemoveStream, (uint64_t)j) * (double)(j + 1));
    if (t > j) t = j;
    if (!pick.insert(t).second) pick.insert(j);
  }
  if (L->removed.empty()) L->removed.assign((size_t)L->total, 0);
  for (int64_t c : pick) L->removed[(size_t)(c * L->cell.n_atoms + a)] = 1;
  return TBK_OK;
}

int tbk_lattice_get_removed(tbk_lattice L, uint8_t* out) {
  if (!L || !out) return fail(TBK_ERR_INVALID, "tbk_lattice_get_removed: null argument");
  if (L->removed.empty()) std::memset(out, 0, (size_t)L->total);
  else std::memcpy(out, L->removed.data(), (size_t)L->total);
  return TBK_OK;
}

int tbk_lattice_kept_number(tbk_lattice L, int64_t* n) {
  if (!L || !n) return fail(TBK_ERR_INVALID, "tbk_lattice_kept_number: null argument");
  int64_t k = L->total;
  if (!L->removed.empty()) { k = 0; for (auto r : L->removed) k += r ? 0 : 1; }
  *n = k;
  return TBK_OK;
}

int tbk_random_phase_kets(int32_t n, int32_t R, uint64_t seed, double* kets) {
  if (n < 1 || R < 1 || !kets) return fail(TBK_ERR_INVALID, "tbk_random_phase_kets: bad argument");
  const double inv = 1.0 / std::sqrt((double)n);
  const double two_pi = 6.283185307179586476925286766559;
  for (int32_t r = 0; r < R; ++r)
    for (int32_t i = 0; i < n; ++i) {
      double th = two_pi * tbk::u01(seed, (uint64_t)r, (uint64_t)i);
      kets[2 * ((int64_t)r * n + i)] = std::cos(th) * inv;
      kets[2 * ((int64_t)r * n + i) + 1] = std::sin(th) * inv;
    }
  return TBK_OK;
}

}  // extern "C"
