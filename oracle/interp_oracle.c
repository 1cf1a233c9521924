/*
 * C restatement of the reference table interpolation — TEST / CPU-BASELINE
 * INFRASTRUCTURE ONLY (used by tests and by the CPU-baseline leg of bench.py,
 * never by the product library).
 *
 * Follows mmuckley/torchkbnufft table mode operation by operation:
 *   tm   = omega / (fl(1/K) * fl(2 pi))                 torchkbnufft/_nufft/interp.py:171
 *   base = 1 + floor(tm - J/2)                          interp.py:177
 *   bin  = rint((tm - (base + j)) * L) + floor(J*L/2)   interp.py:129-132, 174
 *   coef = prod_d table_d[bin_d]  (conj for adjoint)    interp.py:138-144
 *   idx  = sum_d ((base_d + j_d) mod K_d) * prod K[d+1:] interp.py:146-148
 *   forward: y = sum over offsets (in itertools.product order) of coef * x[idx],
 *            then * exp(i sum_d omega_d n_shift_d)      interp.py:185-203
 *   adjoint: x[idx] += conj(coef) * conj(phase) * y, one (batch, coil) plane per
 *            thread as the reference forks over planes  interp.py:406-462, 680-724
 * Compile with -ffp-contract=off so no step is fused into an FMA.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXD 3
#define MAXJ 16

#define DEFINE_ORACLE(R, SUF)                                                                                   \
  typedef struct {                                                                                              \
    int base[MAXD];                                                                                             \
    R tm[MAXD];                                                                                                 \
  } pt_##SUF;                                                                                                   \
                                                                                                                \
  static void point_setup_##SUF(int ndim, const int64_t* K, const int* J, const R* omega, int64_t M, int64_t m, \
                                pt_##SUF* p) {                                                                  \
    for (int d = 0; d < ndim; ++d) {                                                                            \
      R one = (R)1, twopi = (R)6.283185307179586476925286766559;                                                \
      R gam = (one / (R)K[d]) * twopi;                                                                          \
      R tm = omega[d * M + m] / gam;                                                                            \
      R half = (R)J[d] / (R)2;                                                                                  \
      R sh = tm - half;                                                                                         \
      p->tm[d] = tm;                                                                                            \
      p->base[d] = 1 + (int)floor(sh);                                                                          \
    }                                                                                                           \
  }                                                                                                             \
                                                                                                                \
  /* coefficient (re, im) and flat index for neighbour offset `off` */                                          \
  static void coef_idx_##SUF(int ndim, const int64_t* K, const int* J, const int* L, const R* const* tab,       \
                             const pt_##SUF* p, const int* off, int conj, R* cre, R* cim, int64_t* idx) {       \
    R re = (R)1, im = (R)0;                                                                                     \
    int64_t flat = 0;                                                                                           \
    for (int d = 0; d < ndim; ++d) {                                                                            \
      int g = p->base[d] + off[d];                                                                              \
      R diff = p->tm[d] - (R)g;                                                                                 \
      R s = diff * (R)L[d];                                                                                     \
      int64_t k = (int64_t)rint(s) + ((int64_t)J[d] * L[d]) / 2;                                                \
      if (k < 0) k = 0;                                                                                         \
      if (k > (int64_t)J[d] * L[d]) k = (int64_t)J[d] * L[d];                                                   \
      R tr = tab[d][2 * k], ti = tab[d][2 * k + 1];                                                             \
      if (conj) ti = -ti;                                                                                       \
      R nr = re * tr - im * ti;                                                                                 \
      R ni = re * ti + im * tr;                                                                                 \
      re = nr;                                                                                                  \
      im = ni;                                                                                                  \
      int64_t w = g % K[d];                                                                                     \
      if (w < 0) w += K[d];                                                                                     \
      flat = flat * K[d] + w;                                                                                   \
    }                                                                                                           \
    *cre = re;                                                                                                  \
    *cim = im;                                                                                                  \
    *idx = flat;                                                                                                \
  }                                                                                                             \
                                                                                                                \
  static int next_offset_##SUF(int ndim, const int* J, int* off) {                                             \
    for (int d = ndim - 1; d >= 0; --d) {                                                                       \
      if (++off[d] < J[d]) return 1;                                                                            \
      off[d] = 0;                                                                                               \
    }                                                                                                           \
    return 0;                                                                                                   \
  }                                                                                                             \
                                                                                                                \
  static void phase_##SUF(int ndim, const R* omega, int64_t M, int64_t m, const R* nshift, R* c, R* s) {       \
    R a = omega[m] * nshift[0];                                                                                 \
    for (int d = 1; d < ndim; ++d) {                                                                            \
      R t = omega[d * M + m] * nshift[d];                                                                       \
      a = a + t;                                                                                                \
    }                                                                                                           \
    *c = cos(a);                                                                                                \
    *s = sin(a);                                                                                                \
  }                                                                                                             \
                                                                                                                \
  void tkbn_oracle_interp_fwd_##SUF(int ndim, const int64_t* K, const int* J, const int* L, const R* nshift,   \
                                    const R* const* tab, const R* grid, int64_t B, int64_t C, const R* omega,  \
                                    int64_t M, R* kdata, int nthreads) {                                        \
    int64_t G = 1;                                                                                              \
    for (int d = 0; d < ndim; ++d) G *= K[d];                                                                   \
    _Pragma("omp parallel for schedule(static) num_threads(nthreads)") for (int64_t m = 0; m < M; ++m) {       \
      pt_##SUF p;                                                                                               \
      point_setup_##SUF(ndim, K, J, omega, M, m, &p);                                                           \
      for (int64_t bc = 0; bc < B * C; ++bc) {                                                                  \
        kdata[2 * (bc * M + m)] = 0;                                                                            \
        kdata[2 * (bc * M + m) + 1] = 0;                                                                        \
      }                                                                                                         \
      int off[MAXD] = {0, 0, 0};                                                                                \
      do {                                                                                                      \
        R cr, ci;                                                                                               \
        int64_t idx;                                                                                            \
        coef_idx_##SUF(ndim, K, J, L, tab, &p, off, 0, &cr, &ci, &idx);                                         \
        for (int64_t bc = 0; bc < B * C; ++bc) {                                                                \
          R xr = grid[2 * (bc * G + idx)], xi = grid[2 * (bc * G + idx) + 1];                                   \
          R pr = cr * xr - ci * xi, pi = cr * xi + ci * xr;                                                     \
          kdata[2 * (bc * M + m)] += pr;                                                                        \
          kdata[2 * (bc * M + m) + 1] += pi;                                                                    \
        }                                                                                                       \
      } while (next_offset_##SUF(ndim, J, off));                                                               \
      R c, s;                                                                                                   \
      phase_##SUF(ndim, omega, M, m, nshift, &c, &s);                                                           \
      for (int64_t bc = 0; bc < B * C; ++bc) {                                                                  \
        R yr = kdata[2 * (bc * M + m)], yi = kdata[2 * (bc * M + m) + 1];                                       \
        kdata[2 * (bc * M + m)] = yr * c - yi * s;                                                              \
        kdata[2 * (bc * M + m) + 1] = yr * s + yi * c;                                                          \
      }                                                                                                         \
    }                                                                                                           \
  }                                                                                                             \
                                                                                                                \
  void tkbn_oracle_interp_adj_##SUF(int ndim, const int64_t* K, const int* J, const int* L, const R* nshift,   \
                                    const R* const* tab, const R* kdata, int64_t B, int64_t C, const R* omega, \
                                    int64_t M, R* grid, int nthreads) {                                         \
    int64_t G = 1;                                                                                              \
    for (int d = 0; d < ndim; ++d) G *= K[d];                                                                   \
    memset(grid, 0, sizeof(R) * 2 * (size_t)(B * C * G));                                                      \
    _Pragma("omp parallel for schedule(dynamic, 1) num_threads(nthreads)") for (int64_t bc = 0; bc < B * C;    \
                                                                                ++bc) {                        \
      R* plane = grid + 2 * bc * G;                                                                             \
      for (int64_t m = 0; m < M; ++m) {                                                                         \
        pt_##SUF p;                                                                                             \
        point_setup_##SUF(ndim, K, J, omega, M, m, &p);                                                         \
        R c, s;                                                                                                 \
        phase_##SUF(ndim, omega, M, m, nshift, &c, &s);                                                         \
        R yr = kdata[2 * (bc * M + m)], yi = kdata[2 * (bc * M + m) + 1];                                       \
        R vr = yr * c + yi * s, vi = yi * c - yr * s;                                                           \
        int off[MAXD] = {0, 0, 0};                                                                              \
        do {                                                                                                    \
          R cr, ci;                                                                                             \
          int64_t idx;                                                                                          \
          coef_idx_##SUF(ndim, K, J, L, tab, &p, off, 1, &cr, &ci, &idx);                                       \
          plane[2 * idx] += cr * vr - ci * vi;                                                                  \
          plane[2 * idx + 1] += cr * vi + ci * vr;                                                              \
        } while (next_offset_##SUF(ndim, J, off));                                                             \
      }                                                                                                         \
    }                                                                                                           \
  }

DEFINE_ORACLE(float, f32)
DEFINE_ORACLE(double, f64)

int tkbn_oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
