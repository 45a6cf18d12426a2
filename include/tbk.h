/*
 * tbk.h — C ABI of the GB300 (sm_103a) kernel-polynomial library for
 * chenzehan/tight_binding.
 *
 * Plain C: pointers, sizes and int status codes; no CUDA or C++ types in the
 * signatures (streams are passed as `void*` holding a cudaStream_t; NULL is the
 * legacy default stream).  Every entry point returns TBK_OK (0) or an error
 * code, and tbk_last_error() gives the message of the calling thread's last
 * failure.  There is no CPU fallback: without a usable GPU the compute entry
 * points fail with TBK_ERR_CUDA.
 *
 * Layout conventions (those of the reference, which uses Eigen):
 *   - complex numbers are interleaved (re, im) doubles (std::complex<double>);
 *   - a block of R vectors is an N x R column-major complex matrix, ld = N
 *     (Eigen::MatrixXcd), element (i, r) at [2*(r*N + i)];
 *   - sparse matrices are compressed CSC with int32 indices, inner (row)
 *     indices sorted within each column (Eigen::SparseMatrix<Scalar>,
 *     outerIndexPtr / innerIndexPtr / valuePtr).
 *
 * Each declaration names the reference interface it replaces (file:line, paths
 * relative to the reference project root).
 */
#ifndef TBK_H
#define TBK_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  TBK_OK = 0,
  TBK_ERR_INVALID = 1,      /* bad argument (the reference printed to cerr)      */
  TBK_ERR_CUDA = 2,         /* CUDA runtime error / no device                    */
  TBK_ERR_NOMEM = 3,        /* device allocation failed                          */
  TBK_ERR_UNSUPPORTED = 4,  /* valid request outside what is implemented        */
  TBK_ERR_TIMEOUT = 5,      /* bounded device wait gave up                       */
  TBK_ERR_BUDGET = 6        /* request exceeds the admission (HBM) budget        */
};
const char* tbk_last_error(void);
int tbk_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int tbk_device_count(void);

/* ------------------------------------------------------------ precision */
enum {
  TBK_PREC_FP64 = 0,        /* complex128 recursion, FP64 H: the plain drop-in   */
  TBK_PREC_MIXED = 1,       /* complex64 recursion, FP32 H, FP64 moment sums     */
  TBK_PREC_DD = 2           /* double-float recursion (FP32 hi + lo pairs, ~48
                               bits) on the FP32 pipe: FP64-class accuracy at
                               memory speed on GB300's slow FP64 pipe          */
};
enum {
  TBK_FLAG_PREC_MASK = 0xF,
  TBK_FLAG_DOUBLING = 1 << 4,     /* bras == kets: mu_2n, mu_2n+1 from <v_n|v_n>,
                                     <v_n+1|v_n> — half the recursion steps      */
  TBK_FLAG_DEVICE_PTRS = 1 << 5,  /* bras/kets/mu are device pointers           */
  TBK_FLAG_NO_L2_ZIGZAG = 1 << 6, /* keep every step's sweep ascending          */
  TBK_FLAG_STAGED = 1 << 7,       /* TMA-staged warp-specialised step kernel      */
  TBK_FLAG_TWO_STEP = 1 << 8,     /* mixed doubling: two recursion steps per pass
                                     over memory (temporal blocking; 1/3 less DRAM
                                     traffic, but the gathers are latency-bound on
                                     GB300 and it measures slower, so opt-in)     */
  TBK_FLAG_NO_GRAPH = 1 << 9,     /* never replay the recursion as a CUDA graph
                                     (small single-chunk plans capture their
                                     launch sequence on the second identical run) */
  TBK_FLAG_PERSISTENT = 1 << 10,  /* small single-chunk plans: the whole recursion
                                     in one launch.  Complex64 vectors of an H~
                                     with row classes that fit one SM: one CTA
                                     per vector (4,096 sites, R = 8: 0.40 ms
                                     against 0.63 ms for per-step launches).
                                     Otherwise one thread-block cluster per
                                     vector holding its rows and H~ in shared
                                     memory (slower in FP64).  Opt-in: the
                                     moment sums are grouped per vector      */
  TBK_FLAG_NO_CACHE = 1 << 11     /* tbk_cheb_braket_*: build and free the matrix
                                     and plan in this call instead of reusing
                                     the cached ones                           */
};

/* =========================================================================
 * Unit cell (host model).  Replaces UnitCell<Dim> construction and hopping
 * management, TB/unit_cell.h:69-71, 188-256, 527-547, 678-707.
 * ========================================================================= */
typedef struct tbk_cell_s* tbk_cell;

/* UnitCell(lattice_vectors, atoms), TB/unit_cell.h:188-210.
 * lattice_vectors: dim rows of 3 doubles; positions: n_atoms rows of 3. */
int tbk_cell_create(tbk_cell* out, int32_t dim, const double* lattice_vectors,
                    int32_t n_atoms, const char* const* names, const double* positions);
int tbk_cell_copy(tbk_cell* out, tbk_cell src);
void tbk_cell_destroy(tbk_cell cell);
/* add_hopping(from, to, lattice_vector, t), TB/unit_cell.h:212-228 (+534-547). */
int tbk_cell_add_hopping(tbk_cell cell, const char* from, const char* to,
                         const int32_t* lattice_vector, double t_re, double t_im);
/* add_hopping(from, n_NN, t), TB/unit_cell.h:230-256; nn = 0 is On_Site. */
int tbk_cell_add_hopping_nn(tbk_cell cell, const char* from, int32_t nn, double t_re,
                            double t_im);
/* get_atom_index, TB/unit_cell.h:101. */
int tbk_cell_atom_index(tbk_cell cell, const char* name, int32_t* index);
int tbk_cell_info(tbk_cell cell, int32_t* dim, int32_t* n_atoms, int32_t* n_hops);
/* Canonical hopping table (from >= to), in enumeration order. */
int tbk_cell_get_hoppings(tbk_cell cell, int32_t* from, int32_t* to, int32_t* latv3,
                          double* t2);
/* bases: 3 x dim column-major (Eigen bases); positions: n_atoms x 3. */
int tbk_cell_get_geometry(tbk_cell cell, double* bases, double* positions);
/* Number of warnings the last call produced (the reference's cerr messages,
 * e.g. "Hopping already exists", TB/unit_cell.h:536-543). */
int tbk_cell_last_warnings(tbk_cell cell, int32_t* count);

/* =========================================================================
 * Lattice and device Hamiltonian builder.  Replaces PartialLattice<Dim>,
 * TB/lattice.h:22-117, 216-305, 313-377, 446-505.
 * ========================================================================= */
typedef struct tbk_lattice_s* tbk_lattice;

/* PartialLattice(cell, span_size), TB/lattice.h:105-117. */
int tbk_lattice_create(tbk_lattice* out, tbk_cell cell, const int32_t* span);
void tbk_lattice_destroy(tbk_lattice lat);
/* get_total_number, TB/lattice.h:51. */
int tbk_lattice_total_number(tbk_lattice lat, int64_t* n);
/* gauge_field, TB/lattice.h:73: A(r) = G r + c evaluated on the device (covers
 * every uniform field in a linear gauge, e.g. Landau A = (0, B x, 0)). */
int tbk_lattice_set_gauge_linear(tbk_lattice lat, const double* G_rowmajor_3x3,
                                 const double* c3);
/* gauge_field given by its value at every bare site (N x 3, host), for an
 * arbitrary A(r) evaluated by the caller at atom_position(from, i_v). */
int tbk_lattice_set_gauge_sites(tbk_lattice lat, const double* A_sites);
int tbk_lattice_clear_gauge(tbk_lattice lat);
/* set_scalar_field(f), TB/lattice.h:495-505, with f sampled at every bare site
 * (N doubles, host).  Adds zero on-site hoppings to the cell as the reference does. */
int tbk_lattice_set_scalar_sites(tbk_lattice lat, const double* V_sites);
/* set_scalar_field with Anderson disorder V = W (u - 1/2), u ~ U[0,1) keyed by
 * (seed, bare site index); generated on the device. */
int tbk_lattice_set_scalar_disorder(tbk_lattice lat, double W, uint64_t seed);
/* Vacancies (TB/lattice.h:389-464).  Removed sites drop out of the open-boundary
 * Hamiltonian (get_Hamiltonian_sparse) and the position operators; the bare ->
 * compressed index (index_comp_construct) is a device prefix-sum compaction at
 * build time.  set_removed: bare site flags (N, 1 = removed; NULL clears). */
int tbk_lattice_set_removed(tbk_lattice lat, const uint8_t* removed_sites);
/* remove_atoms(atom_name, cells), TB/lattice.h:389-402: `n` lattice vectors
 * (n x Dim int32, row-major); the atom `atom` of each cell is removed.  Unknown
 * atom: TBK_ERR_INVALID "Atom <name> does not exist in the unit cell." */
int tbk_lattice_remove_atoms(tbk_lattice lat, const char* atom, const int32_t* cells, int64_t n);
/* remove_atoms_random(atom_name, n), TB/lattice.h:404-418: `n` distinct cells
 * drawn from a seeded stream (the reference seeds from std::random_device);
 * n > cell number: TBK_ERR_INVALID "The random selection is larger than the
 * total number." */
int tbk_lattice_remove_atoms_random(tbk_lattice lat, const char* atom, int64_t n, uint64_t seed);
/* The current removal flags (N bytes, 1 = removed). */
int tbk_lattice_get_removed(tbk_lattice lat, uint8_t* removed_sites);
/* index_comp construction, TB/lattice.h:446-457: number of kept sites. */
int tbk_lattice_kept_number(tbk_lattice lat, int64_t* n);

/* Device-resident sparse matrix (CSC + sliced-ELL). */
typedef struct tbk_sparse_s* tbk_sparse;

enum {
  TBK_BUILD_SPARSE = 0,          /* get_Hamiltonian_sparse<Scalar>(), TB/lattice.h:262-305 */
  TBK_BUILD_PERIODIC_BARE = 1,   /* get_Hamiltonian_periodic_extend_bare_sparse, :216-258 */
  TBK_BUILD_BARE = 2             /* get_Hamiltonian_bare_sparse<Scalar>(), :347-377       */
};
/* Builds H on the device, bit-exact in structure with the reference's triplet
 * list + setFromTriplets.  extend: per-axis periodic flags (PERIODIC_BARE only). */
int tbk_build_hamiltonian(tbk_sparse* out, tbk_lattice lat, int32_t mode,
                          const int32_t* extend, int32_t is_complex, void* stream);
/* op_position(axis), TB/lattice.h:313-336: the diagonal X as a sparse matrix. */
int tbk_build_position(tbk_sparse* out, tbk_lattice lat, int32_t axis, void* stream);
/* Bond-displacement velocity: the matrix of tbk_build_hamiltonian with every
 * hopping entry (row i, column j) multiplied by scale * (r_i - r_j)_axis taken
 * along the bond itself (the hop's lattice vector), so bonds across a periodic
 * boundary get their short displacement; on-site terms and the scalar field
 * drop out.  With scale = 1/a it equals [X, H~] (op_velocity / the Kubo
 * drivers' X H~ - H~ X, TB/lattice.h:338-345, TB/snippets.h:316-317) on every
 * bond that does not wrap, and stays translation invariant where [X, H~]
 * jumps by the box length.  No factor i, as the reference's commutator. */
int tbk_build_velocity_bond(tbk_sparse* out, tbk_lattice lat, int32_t mode, const int32_t* extend,
                            int32_t is_complex, int32_t axis, double scale, void* stream);
/* Wraps a CSC (Eigen compressed layout).  device_ptrs: arrays already on the GPU. */
int tbk_sparse_from_csc(tbk_sparse* out, int32_t rows, int32_t cols, int64_t nnz,
                        const int32_t* col_ptr, const int32_t* row_idx,
                        const double* values, int32_t is_complex, int32_t device_ptrs,
                        void* stream);
int tbk_sparse_info(tbk_sparse A, int32_t* rows, int32_t* cols, int64_t* nnz,
                    int32_t* is_complex);
/* Row classes of the recursion form (no counterpart in the reference, whose
 * cuSPARSE path always reads column indices).  When every row's off-diagonal
 * entries repeat one of at most 255 lists of (column - row, value) — a lattice
 * Hamiltonian without vacancies whose hoppings are the same in every cell —
 * the recursion kernels compute neighbours from a small per-class table
 * instead of loading the ELL's columns and values.  Examines A once (exact:
 * every row is compared with its class) and returns the class count, 0 when
 * the matrix does not qualify.  The environment variable TBK_NO_CLASSES=1,
 * read when a matrix is first examined, keeps the ELL form (A/B comparisons). */
int tbk_sparse_row_classes(tbk_sparse A, int32_t* n_classes, void* stream);
/* Copies the CSC arrays to host buffers. */
int tbk_sparse_download(tbk_sparse A, int32_t* col_ptr, int32_t* row_idx, double* values,
                        void* stream);
void tbk_sparse_destroy(tbk_sparse A);
/* GreenFunction rescale (H - b I)/a, FP64 on the device; pattern = pattern(H)
 * union diagonal as Eigen's sparse difference gives, TB/lattice.h:550-559. */
int tbk_sparse_rescale(tbk_sparse* out, tbk_sparse H, double a, double b, void* stream);
/* Velocity: v = X H - H X with X = op_position(axis) (values x_i h - h x_j,
 * same pattern as H), TB/lattice.h:338-345 and TB/snippets.h:316-317. */
int tbk_sparse_commutator(tbk_sparse* out, tbk_sparse H, tbk_sparse X, void* stream);
/* Extreme eigenvalues of a Hermitian matrix by `iters` Lanczos steps on the
 * device from seeded random phases (the reference's matrix_spectral_range_sparse,
 * TB/numerical.h:24-46, which uses Spectra on the CPU and refuses > 5,000
 * rows): the extreme Ritz values e_min, e_max and their residual norms
 * (res_min / res_max may be NULL; an eigenvalue lies within that distance). */
int tbk_spectral_range(tbk_sparse A, int32_t iters, uint64_t seed, double* e_min, double* e_max,
                       double* res_min, double* res_max, void* stream);

/* ---------------------------------------------------------------------------
 * Chebyshev expansions applied to vectors
 * ------------------------------------------------------------------------ */
/* out = sum_{k < n_terms} coef_k T_k(H~) kets for R column-major complex128
 * vectors (host, n x R; coef complex, interleaved re/im).  Replaces walking
 * Cheb_first_kind_seq_view (TB/numerical.h:346-361) and summing on the host, as
 * conductivity_test_sawtooth does (TB/snippets.h:173-223).  precision:
 * TBK_PREC_FP64 / TBK_PREC_DD / TBK_PREC_MIXED for the recursion; the sum is
 * accumulated in complex128. */
int tbk_cheb_expand(tbk_sparse Ht, int32_t n_terms, const double* coef, int32_t R, const double* kets, double* out,
                    int32_t precision, void* stream);
/* Cheb_first_kind_seq_view(x, v), TB/numerical.h:346-361: next() yields
 * (i, T_i(H~) v) for i = 0, 1, 2, ... (R column-major complex128 vectors, host
 * in and out; block may be NULL to skip the copy); the two newest blocks stay
 * on the device, one recursion step per call. */
typedef struct tbk_cheb_view_s* tbk_cheb_view;
int tbk_cheb_view_create(tbk_cheb_view* view, tbk_sparse Ht, int32_t R, const double* kets, int32_t precision);
int tbk_cheb_view_next(tbk_cheb_view view, int32_t* index, double* block, void* stream);
void tbk_cheb_view_destroy(tbk_cheb_view view);
/* Delta-projection coefficients of conductivity_test_sawtooth (TB/snippets.h:
 * 175, 194-202): coef_k = a_d(k) T_k(e), a_d(0) = 1, a_d(k>0) = 2, for
 * k = 0 .. N (N + 1 complex values). */
int tbk_cheb_coef_delta(double e, int32_t N, double* coef);
/* exp(-i H t) for H = a H~ + b: coef_k = exp(-i b t) (2 - delta_k0) (-i)^k J_k(a t). */
int tbk_cheb_coef_evolution(double a, double b, double t, int32_t n_terms, double* coef);
/* Number of terms after which |J_k(a t)| stays below tol. */
int tbk_cheb_evolution_terms(double a, double t, double tol, int32_t* n_terms);

/* ---------------------------------------------------------------------------
 * Moment files: binary replacement of the text dumps of utils::output_to_file
 * (TB/utils.h:42-69) and generate_V_moments' V_moments.txt (TB/snippets.h:
 * 504-517).  One file = a fixed 256-byte little-endian header, then rows x cols
 * values (doubles; complex: interleaved re/im) in row-major order.  The header
 * carries what is needed to reuse the moments (bounds, R, seed, kernel,
 * precision) and an FNV-1a 64 checksum of the data bytes, checked on load.
 * ------------------------------------------------------------------------ */
enum {
  TBK_MOMENTS_DOS = 1,      /* mu_n, n < rows (cols = 1), real                 */
  TBK_MOMENTS_MU_NM = 2,    /* mu_nm (rows x cols), complex (Kubo)             */
  TBK_MOMENTS_V_NM = 3      /* V_nm, upper triangle (rows x cols), real        */
};
typedef struct tbk_moments_header {
  char magic[8];            /* "TBKMOM" 0 1                                   */
  int32_t version;          /* 1                                               */
  int32_t kind;             /* TBK_MOMENTS_*                                   */
  int32_t rows, cols;
  int32_t is_complex;
  int32_t R;                /* random vectors summed                           */
  int32_t precision;        /* TBK_PREC_* of the recursion                     */
  int32_t kernel;           /* TBK_KERNEL_* applied, -1 = raw moments         */
  uint64_t seed;
  double e_min, e_max;      /* spectral bounds of H~ = (H - b)/a               */
  double kernel_p0, kernel_p1;
  int64_t n_sites;
  uint64_t checksum;        /* FNV-1a 64 of the data bytes (written by save)   */
  char label[160];          /* free text (model, lattice), NUL-terminated      */
} tbk_moments_header;
/* Writes header + data (the magic, version and checksum are filled in). */
int tbk_moments_save(const char* path, const tbk_moments_header* header, const double* data);
/* Reads the header only. */
int tbk_moments_load_header(const char* path, tbk_moments_header* header);
/* Reads header and data; capacity in doubles.  TBK_ERR_INVALID on a bad magic,
 * a short file, too small a buffer or a checksum mismatch. */
int tbk_moments_load(const char* path, tbk_moments_header* header, double* data, int64_t capacity);

/* =========================================================================
 * Chebyshev (KPM) moments.
 * ========================================================================= */
/* Drop-in for cuda::Cheb_first_kind_seq_braket, real M overload,
 * TB/numerics_cuda.cuh:10-11 / TB/numerics_cuda.cu:190-255: host CSC (square,
 * compressed), bras/kets N x R column-major complex128; mu_out[k] =
 * Re tr(bras^dagger T_k(M) kets), k < n.  n < 2 -> TBK_ERR_INVALID (the
 * reference returns an empty vector).  flags: TBK_PREC_* | TBK_FLAG_DOUBLING
 * (doubling needs bras == kets, same pointer) | TBK_FLAG_NO_CACHE.
 * Every call uploads the CSC arrays and compares them on the device with the
 * previous call's; an identical matrix reuses its device form (ELL, row
 * classes) and the recursion plan of the same R and flags (work blocks, the
 * captured launch graph), which the reference rebuilds per call
 * (TB/numerics_cuda.cu:199-222).  The cache keeps that device memory after the
 * call (about the matrix plus three vector blocks); tbk_cheb_braket_release
 * frees it.  Calls are serialised by a lock. */
int tbk_cheb_braket_real(int32_t n_rows, int64_t nnz, const int32_t* col_ptr,
                         const int32_t* row_idx, const double* values, int32_t n,
                         const double* bras, const double* kets, int32_t R, int32_t flags,
                         double* mu_out);
/* Complex M overload, TB/numerics_cuda.cuh:12-13 / TB/numerics_cuda.cu:266-323. */
int tbk_cheb_braket_complex(int32_t n_rows, int64_t nnz, const int32_t* col_ptr,
                            const int32_t* row_idx, const double* values, int32_t n,
                            const double* bras, const double* kets, int32_t R,
                            int32_t flags, double* mu_out);
/* Frees the matrix and plans cached by tbk_cheb_braket_* (no counterpart in
 * the reference, which keeps nothing between calls). */
void tbk_cheb_braket_release(void);
/* Polls a bounded device wait of the TMA-staged step kernel (TBK_FLAG_STAGED)
 * makes before it gives up, records an error and lets the call return
 * TBK_ERR_TIMEOUT; polls < 0 restores the default (2^24), 0 gives up at once.
 * No counterpart in the reference (its kernels have no waits): it exists so a
 * test can drive the failure path without hanging the GPU.  Copies already in
 * flight are always waited for with the default limit. */
int tbk_set_wait_limit(int64_t polls);

/* Resident solver: H~ and the recursion state stay on the device between runs.
 * Replaces the per-call upload/alloc of TB/numerics_cuda.cu:199-222. */
typedef struct tbk_kpm_s* tbk_kpm;
int tbk_kpm_create(tbk_kpm* out, tbk_sparse Ht, int32_t R, int32_t flags);
/* mu_out (host unless TBK_FLAG_DEVICE_PTRS in the plan's flags). */
int tbk_kpm_run(tbk_kpm plan, int32_t n_mom, const double* bras, const double* kets,
                double* mu_out, void* stream);
/* DoS moments with device-generated random-phase kets (bras = kets),
 * TB/numerical.h:120-122 + TB/functions.h:22-23; seed keys (seed, vector, site). */
int tbk_kpm_run_random(tbk_kpm plan, int32_t n_mom, uint64_t seed, double* mu_out,
                       void* stream);
/* Device time of the recursion kernels of the last run (CUDA events on the
 * launching stream), number of recursion launches and algorithmic DRAM bytes
 * per launch. */
int tbk_kpm_last_timing(tbk_kpm plan, double* ms_recursion, int32_t* launches,
                        double* bytes_per_launch);
void tbk_kpm_destroy(tbk_kpm plan);

/* Random-phase kets exp(2 pi i u)/sqrt(N) (N x R column-major complex128, host),
 * the seeded replacement of bases_of_uniform_ampl_with_random_phases,
 * TB/numerical.h:120-122.  Host function (no GPU needed). */
int tbk_random_phase_kets(int32_t n, int32_t R, uint64_t seed, double* kets);

/* =========================================================================
 * Kernels and reconstruction (FP64 on the device).
 * ========================================================================= */
enum { TBK_KERNEL_DIRICHLET = 0, TBK_KERNEL_FEJER = 1, TBK_KERNEL_LORENTZ = 2,
       TBK_KERNEL_JACKSON = 3, TBK_KERNEL_LANCZOS = 4, TBK_KERNEL_WANG_ZUNGER = 5 };
/* expn_coef_alpha_seq(z, n), TB/numerical.h:304-316: the Chebyshev
 * coefficients of the resolvent, 1/(z - x) = sum_k alpha_k(z) T_k(x), n complex
 * values (interleaved re/im, host math). */
int tbk_expn_coef_alpha_seq(double z_re, double z_im, int32_t n, double* alpha);
/* kernel_seq(N, kernel), TB/numerical.h:393-447.  p0/p1: lambda (Lorentz),
 * M (Lanczos), alpha/beta (Wang-Zunger).  g_out: N doubles, host. */
int tbk_kernel_seq(int32_t kind, int32_t N, double p0, double p1, double* g_out);
/* GreenFunctionImag::operator()(z) = sum_n g_n Im(alpha_n(z)) mu_n for each z,
 * TB/lattice.h:618-624 with TB/numerical.h:304-316.  z: 2*n_z doubles. */
int tbk_green_imag_eval(int32_t n, const double* g, const double* mu, int32_t n_z,
                        const double* z, double* out, void* stream);
/* GreenFunctionImag::fft(upsample): DCT-III of g*mu at x_k = cos((k+1/2)pi/N')
 * times 1/sqrt(1-x^2), N' = n*upsample (moments past n are zero),
 * TB/lattice.h:625-640.  E_out, val_out: N' doubles. */
int tbk_green_imag_fft(int32_t n, const double* g, const double* mu, int32_t upsample,
                       double* E_out, double* val_out, void* stream);
/* density_of_states_seq's last stage, TB/functions.h:26-30: rho(e) =
 * -f(e)/(R pi) on a list of (already rescaled) energies. */
int tbk_dos_from_moments(int32_t n, const double* mu, int32_t kernel_kind, double p0,
                         double p1, double R, int32_t n_e, const double* e, double* rho,
                         void* stream);

/* =========================================================================
 * Kubo conductivities from double-Chebyshev moments.
 * ========================================================================= */
enum {
  TBK_MU_CUDA_CORE = 0,             /* mu_nm GEMM on CUDA cores (FP32 chunks, FP64 sums) */
  TBK_MU_TENSOR = 1,                /* mu_nm GEMM on tcgen05 (split TF32)               */
  TBK_MU_MIXED_RECURSION = 2,       /* complex64 recursion for the stored blocks (FP32
                                       H~); default: complex128 recursion, FP64 H~      */
  TBK_MU_DD_RECURSION = 4,          /* double-float recursion for the stored blocks     */
  TBK_MU_FUSED_OPS = 8,             /* form the output operator's products inside the
                                       recursion step when it shares H~'s sparsity (as
                                       commutators do): same stored bits, one pass per
                                       block instead of two; opt-in: the wider step holds
                                       more registers and measured no faster            */
  TBK_MU_BOTH_SIDES = 16,           /* with TBK_MU_FUSED_OPS: run the left and right
                                       recursions as one of twice the width (same bits;
                                       opt-in, measured no faster)                      */
  TBK_MU_FP64_BLOCKS = 32           /* the FP64 reference form: stored blocks kept in
                                       complex128 and mu_nm formed by an FP64 CUDA-core
                                       GEMM (twice the block memory, FP64-pipe bound);
                                       ignores TBK_MU_TENSOR, FUSED_OPS, BOTH_SIDES     */
};
/* mu_mn = sum_{sites,r} conj(aL_m) aR_n with aL_m = g_m AL T_m(H~) BL |r>,
 * aR_n = g_n AR T_n(H~) BR |r> (NULL operator = identity), m, n < M: the stored
 * Chebyshev blocks of TB/numerical.h:333-344 contracted as in TB/snippets.h:
 * 337-342 (Bastin: AL=BL=1, AR=v_x, BR=v_y), :225-260 (Greenwood: AL=BL=v_x)
 * and :491-518 (generate_V_moments).  Blocks are complex64 in HBM; R vectors
 * are processed in chunks so both sides fit block_budget_gb (<= 0: 60% of the
 * free device memory).
 * kets: host N x R column-major complex128, or NULL for seeded random phases.
 * kernel: TBK_KERNEL_* with parameters kp0/kp1 (g_m).  flags: TBK_MU_*.
 * mu_out: host M x M complex128, row m = left index.
 * Stores and work blocks of at most 16 GB come from a per-device pool that
 * keeps them for the next call (tbk_kubo_release returns them); larger ones
 * are allocated and freed in the call. */
int tbk_kubo_mu(tbk_sparse Ht, tbk_sparse AL, tbk_sparse BL, tbk_sparse AR, tbk_sparse BR, int32_t M,
                int32_t R, uint64_t seed, const double* kets, int32_t kernel_kind, double kp0,
                double kp1, int32_t flags, double block_budget_gb, double* mu_out, void* stream);
/* Returns the memory tbk_kubo_mu's pool keeps on the current device (no
 * counterpart in the reference).  Calls in flight keep theirs. */
int tbk_kubo_release(void);
/* Device time of the last tbk_kubo_mu call in this process (CUDA events on its
 * stream): building the stored blocks, the mu GEMM (+ split-K reduction), the
 * real flops of the GEMM products issued (3 split-TF32 terms on the tensor
 * path), the algorithmic DRAM bytes of the block phase (work vectors read and
 * written, matrix per pass, complex64 stores), and the number of vector chunks. */
int tbk_kubo_last_timing(double* ms_blocks, double* ms_gemm, double* gemm_flops, double* block_bytes,
                         int32_t* chunks);
/* mu_mn = sum_k conj(L_m[k]) R_n[k] for given blocks (host, M x K complex128
 * row-major each, rounded to complex64 on the device): the contraction of
 * TB/snippets.h:337-342 on caller-supplied Chebyshev blocks.  flags: TBK_MU_*
 * (TBK_MU_TENSOR: tcgen05 split-TF32 GEMM).  mu_out: host M x M complex128. */
int tbk_mu_from_blocks(int32_t M, int64_t K, const double* L, const double* Rb, int32_t flags,
                       double* mu_out, void* stream);
/* zeta(e) = sum_mn mu_mn Gamma_mn(e) / (1-e^2)^2 / vol (FP64 on the device),
 * Gamma of TB/snippets.h:343-349; zeta_out: n_eps complex128. */
int tbk_kubo_bastin_zeta(int32_t M, const double* mu, int32_t n_eps, const double* eps, double vol,
                         double* zeta_out, void* stream);
/* sigma(e) = -sum_mn Re(mu_mn) a_m a_n T_m(e) T_n(e) / (1-e^2) / R, the
 * Kubo-Greenwood spectrum of TB/snippets.h:245-260 (FP64 on the device). */
int tbk_kubo_greenwood_sigma(int32_t M, const double* mu, int32_t n_eps, const double* eps, double R,
                             double* sigma_out, void* stream);
/* Cumulative integration of zeta over the N Chebyshev nodes (descending, as the
 * DCT produces them) from E = 0 outward, TB/snippets.h:421-449; writes
 * n_out = N - 2*(N/24) ascending energies with Re / Im integrals. */
int tbk_kubo_bastin_integrate(int32_t N, const double* eps, const double* zeta, double* E_out,
                              double* re_out, double* im_out, int32_t* n_out);

/* =========================================================================
 * Serving: many density-of-states solves advanced together.  No counterpart in
 * the reference, which runs one solve per call (density_of_states_seq,
 * TB/functions.h:15-32, over the moments of TB/numerics_cuda.cu:190-255).
 *
 * A request is a lattice spec plus spectral bounds, M, R, seed and precision.
 * The server copies it at submit, admits it in FIFO order against an HBM
 * budget, builds H~ = (H - b)/a on the device (TBK_BUILD_* as for
 * tbk_build_hamiltonian, a = (e_max - e_min)/2, b = (e_max + e_min)/2) and then
 * advances the running requests together: each round runs `steps_per_round`
 * doubling recursion steps, one launch per (precision, vector width) group and
 * step, packed over all of the group's requests, captured once per group set
 * as a CUDA graph.  Built requests join the running set between rounds while
 * the bytes one step moves stay under `step_gb`.  The random-phase kets are those of tbk_kpm_run_random(seed)
 * and the result is mu_0 .. mu_{M-1} as tbk_kpm_run_random computes them with
 * TBK_FLAG_DOUBLING.  A request's moments do not depend on what else is
 * resident: its sums run in an order fixed by its own size, so a request gives
 * the same bits alone and in any mix.
 * ========================================================================= */
enum { TBK_PENDING = 7 };            /* tbk_server_poll: not finished yet         */
typedef struct tbk_server_s* tbk_server;
typedef struct {
  double budget_gb;                  /* HBM admission cap (<= 0: 120 GB)          */
  int32_t steps_per_round;           /* recursion steps per round (<= 0: 16)      */
  int32_t autotune;                  /* 1: time launch shapes per group at create */
  int32_t max_resident;              /* cap on resident requests (<= 0: 4096)     */
  int32_t result_arena_mb;           /* pinned result arena in MiB (<= 0: 64)     */
  double step_gb;                    /* running set: join built requests while the
                                        bytes one step moves stay below this (<= 0:
                                        2 GB; one request always runs)            */
} tbk_server_config;
typedef struct {
  tbk_lattice lattice;               /* copied at submit                          */
  int32_t build_mode;                /* TBK_BUILD_*                               */
  int32_t extend[3];                 /* periodic axes (TBK_BUILD_PERIODIC_BARE)   */
  int32_t is_complex;                /* Scalar of H (0: double, 1: complex)       */
  int32_t n_mom;                     /* M >= 2                                    */
  int32_t R;                         /* random-phase vectors >= 1                 */
  int32_t precision;                 /* TBK_PREC_MIXED, TBK_PREC_FP64 or _DD      */
  uint64_t seed;
  double e_min, e_max;               /* spectral bounds of H (e_max > e_min)      */
  /* conductivity requests (zero for the DoS moments): */
  int32_t kind;                      /* TBK_REQ_*                                 */
  int32_t axis[2];                   /* position axes a, b of v_a = [x_a, H~]     */
  int32_t kernel;                    /* TBK_KERNEL_* applied to mu_nm             */
  double kernel_p0, kernel_p1;       /* its parameters (Lorentz: lambda)          */
} tbk_request;
/* Request kinds.  DOS: mu_n, n < n_mom (doubling recursion), the moments of
 * density_of_states.  KUBO_BASTIN: g_m g_n mu_nm with mu_nm = <T_m r | v_a T_n v_b r>
 * summed over the R vectors (conductivity_Kubo_Bastin, TB/snippets.h:306-456);
 * KUBO_GREENWOOD: mu_nm = <v_a T_m v_a r | T_n r> (conductivity_spectrum,
 * TB/snippets.h:225-304).  Kubo results are n_mom x n_mom complex128 (row
 * major, 2 n_mom^2 doubles); they run as one tbk_kubo_mu solve on the
 * admission stream while the DoS rounds continue on theirs, with the stored
 * blocks charged to the HBM budget. */
enum { TBK_REQ_DOS = 0, TBK_REQ_KUBO_BASTIN = 1, TBK_REQ_KUBO_GREENWOOD = 2 };
int tbk_server_create(tbk_server* out, const tbk_server_config* cfg);
/* Stops admitting, lets the rounds in flight end, fails what is still queued
 * or resident, frees everything. */
void tbk_server_destroy(tbk_server server);
/* Queues a request; *ticket identifies it.  TBK_ERR_BUDGET when its build peak
 * alone exceeds the budget. */
int tbk_server_submit(tbk_server server, const tbk_request* req, int64_t* ticket);
/* Waits up to wait_ms (>= 0) for the request.  Done: copies the n_mom moments
 * (Kubo requests: the 2 n_mom^2 doubles of mu_nm) to mu_out, times_ms[4] = {queued, build, resident, total} (may be NULL),
 * forgets the ticket and returns TBK_OK.  Not done: TBK_PENDING.  Failed: its
 * status (and forgets the ticket). */
int tbk_server_poll(tbk_server server, int64_t ticket, int32_t wait_ms, double* mu_out,
                    double* times_ms);
/* Footprint of a request as admission charges it: build peak and resident
 * bytes (host arithmetic, no device needed). */
int tbk_request_footprint(const tbk_request* req, int64_t* build_peak_bytes,
                          int64_t* resident_bytes);
/* Counters, out[0 .. n-1] in this order: requests done, failed, rounds, graphs
 * instantiated, GPU busy ms (sum of round durations), algorithmic bytes moved,
 * site-vector updates, step launches, budget bytes, peak reserved bytes,
 * reserved bytes now, build ms (sum), peak resident requests, build overshoot
 * bytes (max over builds of pool high-water minus reservation; <= 0 when
 * admission charged enough). */
int tbk_server_stats(tbk_server server, double* out, int32_t n);
/* Launch shape chosen per group, rows[6*i ..] = {precision, width, form (0:
 * ELL, 1: row classes), grid, L2 prefetch mode (0: none, 1: each tile's own
 * v_s rows at its start, 2: the next wave's tile), ms per step}; returns the
 * number of rows written. */
int tbk_server_tuning(tbk_server server, int32_t max_rows, double* rows);

/* =========================================================================
 * Chebyshev moments without device allocation.  No counterpart in the
 * reference: it serves callers that may not allocate GPU memory while they run
 * (a fixed, fully reserved HBM budget; a host that lends device buffers but
 * forbids allocation; loops where cudaMalloc would synchronise the device).
 * Same result as tbk_cheb_braket_* (FP64 recursion, plain braket moments) for
 * a matrix given in device CSR form (row_ptr[n_rows+1], col_idx, values real or
 * complex interleaved) and device bras/kets (N x R column-major complex128);
 * mu_out is a device array of n_mom doubles, ready when `stream` completes.
 * Work space is a fixed file-scope device array of 32.06 MiB: N * R must not
 * exceed 1,048,576 (larger sizes fail with TBK_ERR_INVALID).  Calls share that
 * array, so calls that overlap on the GPU race.  The CUDA runtime loads device
 * code lazily, so the first call on each device loads the module and reserves
 * the 32.06 MiB array then (it fails with TBK_ERR_CUDA if the device is full):
 * make that call during set-up, before any stream capture.  From then on the
 * array stays reserved on that device until exit and calls allocate and free
 * nothing. */
int tbk_cheb_moments_noalloc(int32_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
                             const double* values, int32_t is_complex, int32_t n_mom,
                             const double* bras, const double* kets, int32_t R, double* mu_out,
                             void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TBK_H */
