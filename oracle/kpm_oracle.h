/*
 * kpm_oracle.h — CPU FP64 oracle for the kernel-polynomial (Chebyshev) path of
 * chenzehan/tight_binding.  TEST INFRASTRUCTURE ONLY: the test-suite, the smoke
 * check and the CPU-baseline leg of bench.py call it as the checker.  Nothing in
 * the product library links or calls this code.
 *
 * Parity status: the reference cannot be compiled or run here (it needs Eigen,
 * FFTW3, Spectra, matplot++ and C++23 library features that are absent, and it
 * ships no tests, fixtures or golden vectors).  This restatement is therefore
 * "parity unpinned" against the reference's own outputs; it is pinned instead
 * against analytic known answers (plane-wave exact traces, nnz counts, the
 * Chebyshev product identities) and against an independent scipy.sparse
 * implementation in tests/.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root; TB/ = tight_binding/).
 *
 * Conventions shared with the GPU library (they define "the same seeded input"):
 *   - complex numbers are interleaved (re, im) doubles;
 *   - dense blocks of R vectors are column-major N x R (Eigen MatrixXcd layout,
 *     ld = N): element (i, r) at [2*(r*N + i)];
 *   - sparse matrices are Eigen-compatible compressed CSC with int32 indices.
 */
#ifndef TB_KPM_ORACLE_H
#define TB_KPM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- seeded inputs (counter-based, replaces std::rand) -------- */
uint64_t tbo_mix64(uint64_t x);
double tbo_u01(uint64_t seed, uint64_t stream, uint64_t idx);
/* |r>_i = exp(i*2*pi*u)/sqrt(n); TB/numerical.h:120-122 (distribution-equivalent). */
void tbo_random_phase_kets(int32_t n, int32_t R, uint64_t seed, double* kets);
/* V_i = W*(u - 1/2), u ~ U[0,1) keyed by bare site index. */
void tbo_uniform_disorder(int32_t n, double W, uint64_t seed, double* v);

/* ---------------- unit cell: n-th nearest-neighbour shell ------------------ */
/* TB/unit_cell.h:678-707.  bases: 3 x dim column-major (bases[c*3 + x]).
 * Writes the shell members (to atom, lattice vector) of atom `from`; returns the
 * count, or -1 when cap is too small. */
int32_t tbo_nn_shell(int32_t dim, const double* bases, int32_t n_atoms,
                     const double* atom_pos, int32_t from, int32_t nn,
                     int32_t* to_out, int32_t* latv_out, int32_t cap);

/* ---------------- lattice -> sparse Hamiltonian --------------------------- */
enum {
  TBO_MODE_SPARSE = 0,          /* get_Hamiltonian_sparse, TB/lattice.h:262-305 */
  TBO_MODE_PERIODIC_BARE = 1,   /* get_Hamiltonian_periodic_extend_bare_sparse, :216-258 */
  TBO_MODE_BARE = 2             /* get_Hamiltonian_bare_sparse, :347-377 */
};
enum { TBO_GAUGE_NONE = 0, TBO_GAUGE_LINEAR = 1, TBO_GAUGE_SITE = 2 };

typedef struct {
  int32_t dim, n_atoms;
  int32_t span[3];
  int32_t extend[3];            /* periodic axes (periodic modes) */
  const double* bases;          /* 3 x dim column-major */
  const double* atom_pos;       /* n_atoms x 3 */
  int32_t n_hops;               /* canonical hopping table, enumeration order */
  const int32_t* hop_from;
  const int32_t* hop_to;
  const int32_t* hop_latv;      /* n_hops x 3 */
  const double* hop_t;          /* n_hops x 2 (re, im) */
  int32_t mode;
  int32_t is_complex;           /* Scalar = Complex (1) or double (0) */
  int32_t gauge_kind;
  const double* gauge_linear;   /* A(r) = G r + c : G row-major 3x3 then c[3] */
  const double* gauge_site;     /* A at every bare site (N x 3) */
  const double* scalar_site;    /* scalar field at every bare site (N) or NULL */
  const int32_t* removed;       /* 1 = removed bare site (N) or NULL */
} tbo_lattice;

int64_t tbo_total_sites(const tbo_lattice* L);
/* Number of rows of the compressed (vacancy-free) index, TB/lattice.h:446-464. */
int64_t tbo_compressed_sites(const tbo_lattice* L);
/* Upper bound on triplets (before duplicate summation). */
int64_t tbo_triplet_bound(const tbo_lattice* L);
/* Builds Eigen-compatible CSC (setFromTriplets semantics: inner indices sorted,
 * duplicates summed in insertion order, explicit zeros kept).  values: nnz
 * doubles (real) or 2*nnz (complex).  Returns nnz, or -1 if cap too small. */
int64_t tbo_build_csc(const tbo_lattice* L, int32_t* col_ptr, int32_t* row_idx,
                      double* values, int64_t cap);
/* Position operator diag, TB/lattice.h:313-336 (CSC with one entry per kept site). */
int64_t tbo_position_diag(const tbo_lattice* L, int32_t axis, double* x_out);

/* ---------------- rescale: (H - b I)/a, pattern U diagonal ------------------ */
/* TB/lattice.h:550-559.  Returns nnz of the result or -1 if cap too small. */
int64_t tbo_rescale_csc(int32_t n, const int32_t* col_ptr, const int32_t* row_idx,
                        const double* values, int32_t is_complex, double a, double b,
                        int32_t* out_col_ptr, int32_t* out_row_idx, double* out_values,
                        int64_t cap);

/* ---------------- velocity: v = X H - H X ---------------------------------- */
/* TB/lattice.h:338-345 and TB/snippets.h:316-317: same pattern as H, values
 * x_i*h - h*x_j.  x: diagonal positions per row. */
void tbo_commutator_values(int32_t n, const int32_t* col_ptr, const int32_t* row_idx,
                           const double* values, int32_t is_complex, const double* x,
                           double* out_values);

/* ---------------- sparse x dense (Eigen column-major semantics) ------------ */
/* y = alpha*M x (+ beta*y0 when y0 != NULL); x, y: N x R column-major complex. */
void tbo_csc_mult(int32_t n, const int32_t* col_ptr, const int32_t* row_idx,
                  const double* values, int32_t is_complex, int32_t R,
                  const double* x, double* y);

/* ---------------- Chebyshev moments (CPU KPM) ------------------------------ */
/* TB/numerical.h:363-381 with trace_braket TB/numerical.h:126-135.
 * mu[k] = Re tr(bras^dagger T_k(M) kets), k < n.  Returns 0, or -1 for n < 2
 * (the GPU path of the reference returns {} there, TB/numerics_cuda.cu:194-197).
 * threads <= 0: all OpenMP threads.  steps_limit > 0 stops after that many
 * recursion steps (used to time a bounded sample). */
int32_t tbo_cheb_moments(int32_t n_rows, const int32_t* col_ptr, const int32_t* row_idx,
                         const double* values, int32_t is_complex, int32_t n_mom,
                         const double* bras, const double* kets, int32_t R,
                         double* mu, int32_t threads, int32_t steps_limit);
/* Re tr(A^dagger B), TB/numerical.h:127-135. */
double tbo_trace_braket(int32_t n, int32_t R, const double* A, const double* B);
/* tr(A^dagger B) complex, TB/numerical.h:136-144. */
void tbo_trace_braket_complex(int32_t n, int32_t R, const double* A, const double* B,
                              double* out2);

/* Stored Chebyshev blocks T_k(M)|v>, k < n_mom: TB/numerical.h:333-344.
 * out: n_mom blocks of N x R complex (column-major), contiguous. */
int32_t tbo_cheb_blocks(int32_t n_rows, const int32_t* col_ptr, const int32_t* row_idx,
                        const double* values, int32_t is_complex, int32_t n_mom,
                        const double* v, int32_t R, double* out);

/* ---------------- kernels TB/numerical.h:393-447 --------------------------- */
enum { TBO_K_DIRICHLET = 0, TBO_K_FEJER = 1, TBO_K_LORENTZ = 2, TBO_K_JACKSON = 3,
       TBO_K_LANCZOS = 4, TBO_K_WANG_ZUNGER = 5 };
void tbo_kernel_seq(int32_t kind, int32_t N, double p0, double p1, double* g);

/* ---------------- reconstruction ------------------------------------------ */
/* alpha_n(z): TB/numerical.h:304-316; z complex. out: 2*n doubles. */
void tbo_expn_coef_alpha_seq(double z_re, double z_im, int32_t n, double* out);
/* f(e) = sum g_n Im(alpha_n(e)) mu_n, TB/lattice.h:618-624 (z complex). */
double tbo_green_imag_eval(int32_t n, const double* g, const double* mu,
                           double z_re, double z_im);
/* DCT-III (FFTW REDFT01) of g*mu times 1/sqrt(1-x^2) at x_k = cos((k+1/2)pi/N),
 * TB/lattice.h:625-640; direct O(N^2) sum.  Nout = n*upsample, moments beyond n
 * are zero. */
void tbo_green_imag_fft(int32_t n, const double* g, const double* mu, int32_t upsample,
                        double* E_out, double* val_out);

/* ---------------- Kubo ------------------------------------------------------ */
/* mu_nm = tr(L_m^dagger R_n) over stored blocks (complex), TB/snippets.h:337-342.
 * L, Rb: M blocks of K complex each (K = N*R).  out: M x M complex row-major
 * (out[2*(m*M + n)]). */
void tbo_mu_nm(int32_t M, int64_t K, const double* L, const double* Rb, double* out);
/* Bastin Gamma_nm(eps) and zeta(eps) = sum mu_nm Gamma_nm / (1-eps^2)^2 / vol,
 * TB/snippets.h:343-349, 400-415.  mu: M x M complex row-major (m = left index). */
void tbo_bastin_zeta(int32_t M, const double* mu, int32_t n_eps, const double* eps,
                     double vol, double* zeta_out);
/* Greenwood: sigma(eps) = -sum_{m,n} mu_mn a_m a_n T_m T_n / (1-eps^2) / R,
 * the diagonal-in-energy form of TB/snippets.h:254-260 (g already folded in mu). */
void tbo_greenwood_sigma(int32_t M, const double* mu, int32_t n_eps, const double* eps,
                         double R, double* sigma_out);

/* Bastin cumulative integration (TB/snippets.h:421-449); returns the count. */
int32_t tbo_bastin_integrate(int32_t N, const double* eps, const double* zeta, double* E, double* re, double* im);

#ifdef __cplusplus
}
#endif
#endif
