/*
 * tkbn_gb300.h — C ABI of the GB300 (sm_103a) table-mode Kaiser-Bessel NUFFT.
 *
 * Plain C: device pointers, sizes and a CUDA stream handle (cudaStream_t passed
 * as void*). No torch types. Every entry point returns an int status
 * (TKBN_OK or a negative TKBN_ERR_*); tkbn_last_error() gives the message of
 * the last failure on the calling thread.
 *
 * Ownership: the caller owns every buffer passed in (inputs, outputs and
 * workspaces). The library allocates nothing except inside
 * tkbn_fft_plan_create (the cuFFT plan or the fused passes' twiddle tables)
 * and tkbn_ragged_plan_create (the merged job lists), which
 * tkbn_fft_plan_destroy and tkbn_ragged_plan_destroy release.
 *
 * Streams: all work is enqueued on the given stream; no entry point
 * synchronises the host, so sequences of calls can be captured in a CUDA
 * graph (except plan creation/destruction).
 *
 * Layouts (row-major, complex = interleaved re/im of the working real type):
 *   image   (B, Ci, N0[, N1[, N2]])   Ci = 1 when smaps are given, else C
 *   smaps   (Bs, C, N0, ...)          Bs = 1 (shared) or B
 *   grid    (B, C, K0[, K1[, K2]])    oversampled Fourier grid
 *   kdata   (B, C, M)
 *   omega   (T, d, M) real            T = 1 (shared trajectory) or B
 *   tables  d pointers, each complex[J_d * L_d + 1]
 *   scaling complex[N0 * N1 * ...]
 *
 * Reference interfaces replaced (mmuckley/torchkbnufft, paths in that project):
 *   tkbn_points_build      sort_data / sort_one_batch   torchkbnufft/_nufft/interp.py:551-584
 *   tkbn_interp_fwd        table_interp                 torchkbnufft/_nufft/interp.py:315-403
 *   tkbn_interp_adj        table_interp_adjoint         torchkbnufft/_nufft/interp.py:587-726
 *   tkbn_interp_grad_omega (none: the reference returns no omega gradient,
 *                           torchkbnufft/_autograd/interp.py:130)
 *   tkbn_fft_and_scale     fft_and_scale (+ SENSE multiply)
 *                          torchkbnufft/_nufft/fft.py:35-76, modules/kbnufft.py:182-183
 *   tkbn_ifft_and_scale    ifft_and_scale (+ coil sum)
 *                          torchkbnufft/_nufft/fft.py:79-118, modules/kbnufft.py:404-405
 *   tkbn_nufft_fwd         kb_table_nufft               torchkbnufft/functional/nufft.py:126-191
 *   tkbn_nufft_adj         kb_table_nufft_adjoint       torchkbnufft/functional/nufft.py:194-260
 *   tkbn_fft_filter        fft_filter                   torchkbnufft/_nufft/fft.py:121-173
 *   tkbn_toep_apply        ToepNufft.forward / toep_batch_loop
 *                          torchkbnufft/modules/kbnufft.py:441-547
 *   tkbn_toep_kernel_assemble  adjoint_flip_and_concat, reflect_conj_concat,
 *                          hermitify  torchkbnufft/_nufft/toep.py:185-307
 *   tkbn_spmat_interp(_adjoint) spmat_interp / spmat_interp_adjoint
 *                          torchkbnufft/_nufft/interp.py:13-85
 *   tkbn_ragged_*          a loop of table_interp / table_interp_adjoint calls
 *                          over independent problems (no single counterpart)
 */
#ifndef TKBN_GB300_H
#define TKBN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TKBN_ABI_VERSION 1

/* status codes */
#define TKBN_OK 0
#define TKBN_ERR_INVALID (-1)     /* bad argument: shape, size, null pointer   */
#define TKBN_ERR_UNSUPPORTED (-2) /* dtype, ndim or numpoints not supported     */
#define TKBN_ERR_CUDA (-3)        /* CUDA runtime error                         */
#define TKBN_ERR_CUFFT (-4)       /* cuFFT error                                */
#define TKBN_ERR_DEVICE (-5)      /* a kernel's own check failed (status word)  */

/* dtypes */
#define TKBN_C64 0  /* complex64: float32 arithmetic  */
#define TKBN_C128 1 /* complex128: float64 arithmetic */

/* FFT normalisation */
#define TKBN_NORM_NONE 0  /* forward unnormalised, inverse without 1/N */
#define TKBN_NORM_ORTHO 1 /* 1/sqrt(prod K) both ways                  */

/* geometry flags */
#define TKBN_TABLES_CONJ_SYMMETRIC 1 /* table[J*L/2 + k] == conj(table[J*L/2 - k]) exactly, for
                                        every dim with J*L even (true for KB tables); the
                                        kernels then read only the first half of each table */
#define TKBN_ADJ_DETERMINISTIC 2     /* layout without split output tiles: every grid cell is
                                        accumulated by one CTA in a fixed order, so the adjoint
                                        is bitwise repeatable (heavy tiles are not spread over
                                        several CTAs). Must be the same in tkbn_points_build
                                        and every call that uses the layout. */
#define TKBN_TABLES_LINEAR_PHASE 8   /* every table is |table[k]| exp(i c (k - J*L/2) / L) to
                                        within float rounding, with c = 2 arg(table[J*L/2 + L/2])
                                        (true for KB tables: the fftshift phase is linear in the
                                        distance); the complex64 2D and 3D gathers and register
                                        adjoints then work with real kernel values and apply the
                                        phases per point and per tile cell or patch cell. Set
                                        only after checking the tables. */
#define TKBN_LAYOUT_FORWARD_ONLY 4   /* layout without the adjoint's per-tile point lists
                                        (smaller workspace, for forward-only callers); an
                                        adjoint on it scans candidates instead (slower). Must
                                        be the same in tkbn_points_build and every call that
                                        uses the layout. */
#define TKBN_ADJ_REUSE_FACTORS 16    /* tkbn_interp_fwd / tkbn_interp_adj / tkbn_nufft_fwd /
                                        tkbn_nufft_adj: the workspace still holds the per-point
                                        table factors that an earlier forward or adjoint call on
                                        it computed, with tables of the same contents (at any
                                        addresses) and the same other flags, so this call
                                        does not recompute them. They depend on the trajectory
                                        and the tables only, not on the grid or k-space data.
                                        No other call writes them; a new tkbn_points_build
                                        invalidates them. A call captured
                                        into a CUDA graph that sets it makes the graph depend
                                        on the factors staying in place; leave it unset there
                                        and the graph recomputes them on every replay. */

/* Operator geometry (one per KbModule). Unused dims (>= ndim) are ignored. */
typedef struct tkbn_geometry {
  int32_t ndim;              /* 1, 2 or 3 */
  int32_t dtype;             /* TKBN_C64 or TKBN_C128 */
  int64_t im_size[3];        /* N_d */
  int64_t grid_size[3];      /* K_d */
  int32_t numpoints[3];      /* J_d, 1..8 */
  int32_t table_oversamp[3]; /* L_d */
  double n_shift[3];         /* fftshift distance per dim */
  int32_t flags;             /* TKBN_TABLES_* bits */
} tkbn_geometry;

/* Sorted-point layout of one trajectory set (built by tkbn_points_build). */
typedef struct tkbn_points_desc {
  int64_t npts;      /* M: points per trajectory */
  int64_t ntraj;     /* 1 (shared by all batch items) or B */
  int32_t tile[3];   /* tile edge per dim in grid cells; 0 = library default */
  int32_t chunk;     /* max points per work item; 0 = library default */
} tkbn_points_desc;

typedef struct tkbn_fft_plan_s* tkbn_fft_plan;

/* ---- library ---------------------------------------------------------- */
int tkbn_abi_version(void);
const char* tkbn_last_error(void);
/* Reads and clears the device status word written by kernels whose internal
 * checks failed (0 = clean). Synchronises the given stream. */
int tkbn_device_status(void* stream, int32_t* status);

/* ---- trajectory layout (K1: bin sort), once per trajectory -------------- */
int tkbn_points_workspace_size(const tkbn_geometry* g, const tkbn_points_desc* p, size_t* bytes);
int tkbn_points_build(const tkbn_geometry* g, const tkbn_points_desc* p, const void* omega,
                      void* workspace, size_t workspace_bytes, void* stream);

/* ---- interpolation ------------------------------------------------------ */
/* kdata = interp(grid): gather of J^d neighbours per point, times the fftshift phase.
 * With 2D complex64 J = 6 layouts of 16 x 14 tiles, and 3D ones of 4 x 8 x 8 tiles with
 * TKBN_TABLES_LINEAR_PHASE, the call fills the workspace's per-point factor scratch as
 * tkbn_interp_adj does (unless TKBN_ADJ_REUSE_FACTORS), and with linear-phase tables
 * the gathers read it, so forward and adjoint calls that share one workspace must be
 * ordered (one stream). */
int tkbn_interp_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                    const void* const* tables, const void* grid, int64_t nbatch, int64_t ncoil,
                    void* kdata, void* stream);
/* grid = interp^H(kdata). grid is fully overwritten (zeroed first). With 2D
 * complex64 J = 6 layouts of 16 x 14 tiles, and 3D ones of 4 x 8 x 8 tiles with
 * TKBN_TABLES_LINEAR_PHASE, the call (forward or adjoint) also fills a per-point
 * scratch region inside the workspace (the table factors; unless
 * TKBN_ADJ_REUSE_FACTORS), so forward and adjoint calls that share one
 * workspace must be ordered (one stream). */
int tkbn_interp_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                    const void* const* tables, const void* kdata, int64_t nbatch, int64_t ncoil,
                    void* grid, void* stream);
/* grad_omega[t,d,m] = Re sum_{b,c} conj(v[b,c,m]) * d/d omega_d (interp(grid))[b,c,m],
 * with the derivative of the KB kernel taken from dtables (d/du of each table
 * entry) and linear interpolation within table bins. grad_omega is overwritten. */
int tkbn_interp_grad_omega(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                           const void* const* tables, const void* const* dtables, const void* grid,
                           const void* v, int64_t nbatch, int64_t ncoil, void* grad_omega, void* stream);

/* Forward interpolation that allocates no device memory (no counterpart in
 * the reference). For callers that cannot allocate device memory after start
 * (a fixed device-memory budget, or a plain-C host holding only raw pointers):
 * the trajectory layout of omega (shared by all batch items, (d, npts)) is
 * built in a library-owned array of TKBN_NOALLOC_SCRATCH_BYTES that each GPU
 * holds until exit; larger trajectories are rejected with TKBN_ERR_INVALID.
 * The first call on a device looks the array up (make it before any stream
 * capture). All calls share the array: calls that overlap on the GPU race. */
#define TKBN_NOALLOC_SCRATCH_BYTES ((size_t)8 << 20)
int tkbn_interp_fwd_noalloc(const tkbn_geometry* g, const void* const* tables, const void* omega, int64_t npts,
                            const void* grid, int64_t nbatch, int64_t ncoil, void* kdata, void* stream);

/* ---- sparse-matrix interpolation ----------------------------------------
 * The interpolation matrix A (nrows k-space points x ncols grid cells,
 * complex of the working type) as CSR (crow[nrows + 1], col[nnz], val[nnz])
 * for the forward and as COO rows (row[nnz]) with the same col/val for the
 * adjoint. x and y hold nplanes (batch x coil) planes of ncols / nrows.
 * Replaces spmat_interp / spmat_interp_adjoint,
 * torchkbnufft/_nufft/interp.py:13-85. */
int tkbn_spmat_interp(int dtype, int64_t nrows, int64_t ncols, const int64_t* crow, const int32_t* col,
                      const void* val, const void* x, int64_t nplanes, void* y, void* stream);
/* x = A^H y; x is fully overwritten. */
int tkbn_spmat_interp_adjoint(int dtype, int64_t nrows, int64_t ncols, int64_t nnz, const int32_t* row,
                              const int32_t* col, const void* val, const void* y, int64_t nplanes, void* x,
                              void* stream);

/* ---- ragged batch (K8): many independent problems per launch ------------
 * No single counterpart in the reference, where each problem is one call of
 * table_interp / table_interp_adjoint (torchkbnufft/_nufft/interp.py:315-403,
 * 587-726). Each problem has its own geometry (grid and image size, tables),
 * trajectory layout (built by tkbn_points_build, ntraj = 1), coil count and
 * device buffers; all share dtype, ndim and numpoints. The plan merges the
 * problems' work into one longest-first job list per stage, so that one
 * launch interpolates every problem; the buffers named here are the ones the
 * launches read and write (a CUDA graph can capture them). */
typedef struct tkbn_ragged_problem {
  tkbn_geometry geom;        /* flags as for the single-problem calls */
  tkbn_points_desc points;   /* ntraj must be 1 */
  const void* workspace;     /* layout of this problem's omega */
  const void* tables[3];     /* per-dim tables of this geometry */
  int64_t ncoil;
  void* grid;                /* (ncoil, K...) */
  void* kdata;               /* (ncoil, M) */
} tkbn_ragged_problem;

typedef struct tkbn_ragged_plan_s* tkbn_ragged_plan;

/* Reads the layouts' work lists (synchronises the device), allocates the
 * merged job lists. Adjoints need grids with K_d >= T_d + J_d - 1. For 2D
 * complex64 register-adjoint layouts it also fills each problem's per-point
 * factor scratch (the one tkbn_interp_adj fills) once, from the problem's
 * tables; while the plan is in use, no other adjoint call may run on those
 * workspaces. */
int tkbn_ragged_plan_create(const tkbn_ragged_problem* problems, int64_t nproblems, tkbn_ragged_plan* plan);
int tkbn_ragged_plan_destroy(tkbn_ragged_plan plan);
/* kdata_p = interp(grid_p) for every problem p, one launch. */
int tkbn_ragged_interp_fwd(tkbn_ragged_plan plan, void* stream);
/* grid_p = interp^H(kdata_p) for every problem p (grids fully overwritten). */
int tkbn_ragged_interp_adj(tkbn_ragged_plan plan, void* stream);

/* ---- FFT stages --------------------------------------------------------- */
/* Plan for nbatch*ncoil transforms of size grid_size: the fused passes' twiddle
 * tables when every grid size has a compile-time plan (2D and 3D), else a cuFFT
 * plan (in place on the grid). */
int tkbn_fft_plan_create(const tkbn_geometry* g, int64_t nbatch, int64_t ncoil, tkbn_fft_plan* plan);
int tkbn_fft_plan_destroy(tkbn_fft_plan plan);

/* grid = FFT(zero_pad(image [* smaps] * scaling)). scaling may be NULL (ones).
 * smaps may be NULL; then image has ncoil channels. */
int tkbn_fft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* smaps,
                       int64_t smaps_batch, const void* scaling, int64_t nbatch, int64_t ncoil, int norm,
                       void* grid, void* stream);
/* image = [sum_c conj(smaps) *] conj(scaling) * crop(IFFT(grid)). grid is used as scratch. */
int tkbn_ifft_and_scale(const tkbn_geometry* g, tkbn_fft_plan plan, void* grid, const void* smaps,
                        int64_t smaps_batch, const void* scaling, int64_t nbatch, int64_t ncoil, int norm,
                        void* image, void* stream);

/* ---- composed operators ------------------------------------------------- */
int tkbn_nufft_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                   tkbn_fft_plan plan, const void* const* tables, const void* scaling, const void* image,
                   const void* smaps, int64_t smaps_batch, int64_t nbatch, int64_t ncoil, int norm,
                   void* grid_scratch, void* kdata, void* stream);
int tkbn_nufft_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* workspace,
                   tkbn_fft_plan plan, const void* const* tables, const void* scaling, const void* kdata,
                   const void* smaps, int64_t smaps_batch, int64_t nbatch, int64_t ncoil, int norm,
                   void* grid_scratch, void* image, void* stream);

/* out = crop(IFFT(kernel * FFT(zero_pad(image)))) per channel. geometry:
 * im_size = image spatial size, grid_size = kernel size. kernel_batch = 1
 * (shared) or ncoil: kernel k filters channel k of every batch item, which is
 * how torch broadcasts a (K, *grid) kernel against a (B, C, *grid) spectrum. */
int tkbn_fft_filter(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel,
                    int64_t kernel_batch, int64_t nbatch, int64_t ncoil, int norm, void* grid_scratch,
                    void* out, void* stream);
/* Toeplitz normal operator with coil maps:
 * out[b] = sum_c conj(s_c) crop(IFFT(kernel * FFT(pad(s_c * image[b])))). */
int tkbn_toep_apply(const tkbn_geometry* g, tkbn_fft_plan plan, const void* image, const void* kernel,
                    int64_t kernel_batch, const void* smaps, int64_t smaps_batch, int64_t nbatch, int64_t ncoil,
                    int norm, void* grid_scratch, void* out, void* stream);
/* Toeplitz kernel assembly (calc_toeplitz_kernel's steps between its adjoint
 * NUFFTs and its FFT, torchkbnufft/_nufft/toep.py:185-307): from
 * parts[P][N0][N1]..., the 2^(ndim-1) adjoint NUFFT images of the weights at
 * the trajectory with dims 1..ndim-1 sign-flipped (pattern p: bit ndim-1-d of
 * p set when dim d is flipped, the order of the reference's recursion),
 * writes out[2 N0][2 N1]... = scale * the Hermitian kernel before its FFT.
 * dtype TKBN_C64 or TKBN_C128; out must not alias parts. */
int tkbn_toep_kernel_assemble(int dtype, int ndim, const int64_t* im_size, const void* parts, double scale,
                              void* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TKBN_GB300_H */
