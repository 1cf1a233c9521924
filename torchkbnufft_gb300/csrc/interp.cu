// K3 (gather), K4 (scatter) and K7 (trajectory-gradient gather) on the
// bin-sorted layout.
//
// One work item = up to `chunk` points whose footprints start inside one grid
// tile. A CTA takes a job (item, batch, coil chunk), stages the tile's patch
// (tile + J-1 halo, wrapped periodically) of Cc coil planes in shared memory,
// and processes the item's points with Cc lanes per point (lane = coil), so the
// J^d table coefficients of a point are shared by its coils and the patch
// reads of one point are spread over distinct banks.
//
// Reference semantics (mmuckley/torchkbnufft):
//   forward  y[b,c,m] = phase_m * sum_j coef_j(m) * X[b,c,idx_j(m)]
//            (table_interp_one_batch, torchkbnufft/_nufft/interp.py:153-203)
//   adjoint  X[b,c,idx_j(m)] += conj(coef_j(m)) * conj(phase_m) * y[b,c,m]
//            (table_interp_adjoint, torchkbnufft/_nufft/interp.py:587-726)
// The separable sums below group the products per dimension; the table bins,
// cell indices and phase argument are computed exactly as the reference does.

#include "geo_host.cuh"
#include "tkbn_common.cuh"

namespace tkbn {

constexpr int kThreads = 256;

template <int D, int JC>
struct JDims {
  static constexpr int N = JC > 0 ? JC : kMaxJ;
};

// Per-point setup shared by all kernels: table factors per dim and the
// point's local footprint origin inside the tile patch.
template <typename R, int D, int JC>
struct PointSetup {
  cplx<R> h[D][JDims<D, JC>::N];
  int local[D];
  R om[D];
  bool ok;
};

template <typename R, int D, int JC>
__device__ __forceinline__ void setup_point(const Geo<R>& geo, const R* __restrict__ coords, int64_t n, int64_t i,
                                            const int* origin, PointSetup<R, D, JC>& ps) {
  ps.ok = true;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const R om = coords[d * n + i];
    ps.om[d] = om;
    R tm;
    int base;
    ps.ok &= base_index<R>(om, geo.gam[d], geo.halfJ[d], &tm, &base);
    const int w = pmod(base, geo.K[d]);
    const int l = w - origin[d];
    ps.ok &= (l >= 0) & (l < geo.T[d]);
    ps.local[d] = l;
    const int J = JC > 0 ? JC : geo.J[d];
#pragma unroll
    for (int j = 0; j < JDims<D, JC>::N; ++j) {
      if (j < J) {
        const int k = table_bin<R>(tm, base + j, geo.Lr[d], geo.center[d], geo.tmax[d]);
        ps.h[d][j] = __ldg(&geo.tab[d][k]);
      } else {
        ps.h[d][j] = mk<R>(0, 0);
      }
    }
  }
}

template <typename R>
__device__ __forceinline__ void job_decode(const Geo<R>& geo, const Item& it, int64_t ntraj, int64_t bb, int* origin,
                                           int64_t* t_out, int64_t* b_out) {
  const int64_t t = it.key / geo.ntiles;
  int rem = (int)(it.key - t * geo.ntiles);
  for (int d = geo.ndim - 1; d >= 0; --d) {
    const int td = rem % geo.ntile[d];
    rem /= geo.ntile[d];
    origin[d] = td * geo.T[d];
  }
  *t_out = t;
  *b_out = ntraj == 1 ? bb : t;
}

// Row decomposition of a patch: a row is P[D-1] cells contiguous in smem and
// (up to the periodic wrap) contiguous in the global grid.
template <typename R, int D>
__device__ __forceinline__ int64_t patch_row_base(const Geo<R>& geo, int row, const int* origin, int64_t* gstride_x) {
  // row -> (c is handled by the caller), outer coordinates
  int64_t flat = 0, stride = geo.K[D - 1];
#pragma unroll
  for (int d = D - 2; d >= 0; --d) {
    const int p = row % geo.P[d];
    row /= geo.P[d];
    flat += (int64_t)pmod(origin[d] + p, geo.K[d]) * stride;
    stride *= geo.K[d];
  }
  *gstride_x = 1;
  return flat;
}

// Stage Cc coil planes of the periodic patch [origin, origin + P) into smem:
// one warp per patch row, lanes along the innermost dimension.
template <typename R, int D>
__device__ __forceinline__ void load_patch(const Geo<R>& geo, const cplx<R>* __restrict__ grid, int64_t plane0,
                                           int64_t gtot, int ncl, int cells, int ps, const int* origin,
                                           cplx<R>* patch) {
  const int PX = geo.P[D - 1];
  const int KX = geo.K[D - 1];
  const int rows_per_plane = cells / PX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int r = warp; r < ncl * rows_per_plane; r += nwarps) {
    const int c = r / rows_per_plane;
    const int rr = r - c * rows_per_plane;
    int64_t sx;
    const cplx<R>* src = grid + (plane0 + c) * gtot + patch_row_base<R, D>(geo, rr, origin, &sx);
    cplx<R>* dst = patch + c * ps + rr * PX;
    for (int px = lane; px < PX; px += 32) {
      int gx = origin[D - 1] + px;
      gx = gx >= KX ? gx - KX * (gx / KX) : gx;
      dst[px] = src[gx];
    }
  }
}

// Add the staged patch into the global grid with vector atomics (cells that
// stayed zero are skipped).
template <typename R, int D>
__device__ __forceinline__ void flush_patch(const Geo<R>& geo, cplx<R>* __restrict__ grid, int64_t plane0,
                                            int64_t gtot, int ncl, int cells, int ps, const int* origin,
                                            const cplx<R>* patch);

template <typename R, int D, int JC>
__device__ __forceinline__ cplx<R> gather_point(const Geo<R>& geo, const PointSetup<R, D, JC>& ps,
                                                const cplx<R>* __restrict__ plane) {
  constexpr int NJ = JDims<D, JC>::N;
  cplx<R> acc = mk<R>(0, 0);
  if (D == 1) {
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (JC > 0 || j < geo.J[0]) acc = cfma<R>(ps.h[0][j], plane[ps.local[0] + j], acc);
  } else if (D == 2) {
    const int P1 = geo.P[1];
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      if (JC > 0 || jy < geo.J[0]) {
        const cplx<R>* row = plane + (ps.local[0] + jy) * P1 + ps.local[1 % D];
        cplx<R> r = mk<R>(0, 0);
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx)
          if (JC > 0 || jx < geo.J[1 % D]) r = cfma<R>(ps.h[1 % D][jx], row[jx], r);
        acc = cfma<R>(ps.h[0][jy], r, acc);
      }
    }
  } else {
    const int P1 = geo.P[1 % D], P2 = geo.P[2 % D];
#pragma unroll 1
    for (int jz = 0; jz < NJ; ++jz) {
      if (JC > 0 || jz < geo.J[0]) {
        cplx<R> sz = mk<R>(0, 0);
#pragma unroll
        for (int jy = 0; jy < NJ; ++jy) {
          if (JC > 0 || jy < geo.J[1 % D]) {
            const cplx<R>* row = plane + ((ps.local[0] + jz) * P1 + ps.local[1 % D] + jy) * P2 + ps.local[2 % D];
            cplx<R> r = mk<R>(0, 0);
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx)
              if (JC > 0 || jx < geo.J[2 % D]) r = cfma<R>(ps.h[2 % D][jx], row[jx], r);
            sz = cfma<R>(ps.h[1 % D][jy], r, sz);
          }
        }
        acc = cfma<R>(ps.h[0][jz], sz, acc);
      }
    }
  }
  return acc;
}

__device__ __forceinline__ void atomic_add_c(float2* p, float2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void atomic_add_c(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
// Global-memory flush: one vector atomic for float2 (sm_90+), two for double.
__device__ __forceinline__ void atomic_add_global(float2* p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_global(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

template <typename R, int D>
__device__ __forceinline__ void flush_patch(const Geo<R>& geo, cplx<R>* __restrict__ grid, int64_t plane0,
                                            int64_t gtot, int ncl, int cells, int ps, const int* origin,
                                            const cplx<R>* patch) {
  const int PX = geo.P[D - 1];
  const int KX = geo.K[D - 1];
  const int rows_per_plane = cells / PX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int r = warp; r < ncl * rows_per_plane; r += nwarps) {
    const int c = r / rows_per_plane;
    const int rr = r - c * rows_per_plane;
    int64_t sx;
    cplx<R>* dst = grid + (plane0 + c) * gtot + patch_row_base<R, D>(geo, rr, origin, &sx);
    const cplx<R>* src = patch + c * ps + rr * PX;
    for (int px = lane; px < PX; px += 32) {
      const cplx<R> v = src[px];
      if (v.x == R(0) && v.y == R(0)) continue;
      int gx = origin[D - 1] + px;
      gx = gx >= KX ? gx - KX * (gx / KX) : gx;
      atomic_add_global(&dst[gx], v);
    }
  }
}

template <typename R, int D, int JC>
__device__ __forceinline__ void scatter_point(const Geo<R>& geo, const PointSetup<R, D, JC>& ps, cplx<R> v,
                                              cplx<R>* plane) {
  constexpr int NJ = JDims<D, JC>::N;
  if (D == 1) {
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (JC > 0 || j < geo.J[0]) atomic_add_c(&plane[ps.local[0] + j], cmulc<R>(v, ps.h[0][j]));
  } else if (D == 2) {
    const int P1 = geo.P[1];
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      if (JC > 0 || jy < geo.J[0]) {
        const cplx<R> vy = cmulc<R>(v, ps.h[0][jy]);
        cplx<R>* row = plane + (ps.local[0] + jy) * P1 + ps.local[1 % D];
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx)
          if (JC > 0 || jx < geo.J[1 % D]) atomic_add_c(&row[jx], cmulc<R>(vy, ps.h[1 % D][jx]));
      }
    }
  } else {
    const int P1 = geo.P[1 % D], P2 = geo.P[2 % D];
#pragma unroll 1
    for (int jz = 0; jz < NJ; ++jz) {
      if (JC > 0 || jz < geo.J[0]) {
        const cplx<R> vz = cmulc<R>(v, ps.h[0][jz]);
#pragma unroll
        for (int jy = 0; jy < NJ; ++jy) {
          if (JC > 0 || jy < geo.J[1 % D]) {
            const cplx<R> vy = cmulc<R>(vz, ps.h[1 % D][jy]);
            cplx<R>* row = plane + ((ps.local[0] + jz) * P1 + ps.local[1 % D] + jy) * P2 + ps.local[2 % D];
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx)
              if (JC > 0 || jx < geo.J[2 % D]) atomic_add_c(&row[jx], cmulc<R>(vy, ps.h[2 % D][jx]));
          }
        }
      }
    }
  }
}

struct Launch {
  const Item* items;
  const int64_t* hdr;  // hdr[0] = number of items
  const int32_t* vals; // sorted -> original flat index t*M + m
  int64_t n;           // ntraj * M
  int64_t M;
  int64_t ntraj;
  int64_t B, C;
  int Cc;              // coils per job (power of two <= 32)
  int ncc;             // coil chunks
  int64_t nbpt;        // batch items per trajectory job (B if shared trajectory else 1)
  int cells;           // prod P
  int ps;              // smem plane stride (elements)
  int64_t gtot;        // prod K
};

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_interp_fwd(Geo<R> geo, Launch a, const R* __restrict__ coords,
                                                         const cplx<R>* __restrict__ grid, cplx<R>* __restrict__ kdata) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * (blockDim.x >> 5);
  const int c = lane % a.Cc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    const int64_t item_idx = job % nitems;
    const int64_t rest = job / nitems;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    const Item it = a.items[item_idx];
    int origin[kMaxDim];
    int64_t t, b;
    job_decode<R>(geo, it, a.ntraj, bb, origin, &t, &b);
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)a.Cc, a.C - c0);
    __syncthreads();
    load_patch<R, D>(geo, grid, b * a.C + c0, a.gtot, ncl, a.cells, a.ps, origin, patch);
    __syncthreads();
    for (int s = warp * ppw + lane / a.Cc; s < it.len; s += ppb) {
      const int64_t i = it.start + s;
      PointSetup<R, D, JC> ps;
      setup_point<R, D, JC>(geo, coords, a.n, i, origin, ps);
      const int64_t m = a.vals[i] - t * a.M;
      if (c < ncl) {
        cplx<R> y;
        if (ps.ok) {
          const cplx<R> acc = gather_point<R, D, JC>(geo, ps, patch + c * a.ps);
          R sn, cs;
          sincos_acc(phase_arg<R, D>(ps.om, geo.nshift), &sn, &cs);
          y = cmul<R>(acc, mk<R>(cs, sn));
        } else {
          y = mk<R>(R(NAN), R(NAN));
        }
        kdata[(b * a.C + c0 + c) * a.M + m] = y;
      }
      if (!ps.ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
  }
}

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_interp_adj(Geo<R> geo, Launch a, const R* __restrict__ coords,
                                                         const cplx<R>* __restrict__ kdata, cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * (blockDim.x >> 5);
  const int c = lane % a.Cc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    const int64_t item_idx = job % nitems;
    const int64_t rest = job / nitems;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    const Item it = a.items[item_idx];
    int origin[kMaxDim];
    int64_t t, b;
    job_decode<R>(geo, it, a.ntraj, bb, origin, &t, &b);
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)a.Cc, a.C - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < ncl * a.ps; idx += blockDim.x) patch[idx] = mk<R>(0, 0);
    __syncthreads();
    for (int s = warp * ppw + lane / a.Cc; s < it.len; s += ppb) {
      const int64_t i = it.start + s;
      PointSetup<R, D, JC> ps;
      setup_point<R, D, JC>(geo, coords, a.n, i, origin, ps);
      const int64_t m = a.vals[i] - t * a.M;
      if (ps.ok && c < ncl) {
        R sn, cs;
        sincos_acc(phase_arg<R, D>(ps.om, geo.nshift), &sn, &cs);
        const cplx<R> v = cmulc<R>(kdata[(b * a.C + c0 + c) * a.M + m], mk<R>(cs, sn));
        scatter_point<R, D, JC>(geo, ps, v, patch + c * a.ps);
      }
      if (!ps.ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
    __syncthreads();
    flush_patch<R, D>(geo, grid, b * a.C + c0, a.gtot, ncl, a.cells, a.ps, origin, patch);
  }
}

// Smooth table lookup for the gradient: linear interpolation of value and
// derivative tables at the exact (unrounded) position.
template <typename R>
__device__ __forceinline__ void lerp_tables(const Geo<R>& geo, int d, R tm, int g, cplx<R>* val, cplx<R>* der) {
  const R s = (tm - (R)g) * geo.Lr[d] + (R)geo.center[d];
  const R fl = floor(s);
  int k = (int)fl;
  R fr = s - fl;
  if (k < 0) {
    k = 0;
    fr = 0;
  }
  if (k >= geo.tmax[d]) {
    k = geo.tmax[d] - 1;
    fr = 1;
  }
  const cplx<R> v0 = __ldg(&geo.tab[d][k]), v1 = __ldg(&geo.tab[d][k + 1]);
  const cplx<R> d0 = __ldg(&geo.dtab[d][k]), d1 = __ldg(&geo.dtab[d][k + 1]);
  *val = mk<R>(v0.x + fr * (v1.x - v0.x), v0.y + fr * (v1.y - v0.y));
  *der = mk<R>(d0.x + fr * (d1.x - d0.x), d0.y + fr * (d1.y - d0.y));
}

// K7: grad_omega[t,d,m] += Re sum_{b,c} conj(v[b,c,m]) * dy/d omega_d, with
// y = phase * sum_j prod_d h_d(u_d) X[idx_j], u_d = tm_d - g_d, tm = omega/gam.
// Uses the patch staging of the forward; one lane per (point, coil), coils
// reduced with warp shuffles, batches with atomics.
template <typename R, int D>
__global__ void __launch_bounds__(kThreads) k_interp_grad(Geo<R> geo, Launch a, const R* __restrict__ coords,
                                                          const cplx<R>* __restrict__ grid,
                                                          const cplx<R>* __restrict__ v, R* __restrict__ grad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * (blockDim.x >> 5);
  const int c = lane % a.Cc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    const int64_t item_idx = job % nitems;
    const int64_t rest = job / nitems;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    const Item it = a.items[item_idx];
    int origin[kMaxDim];
    int64_t t, b;
    job_decode<R>(geo, it, a.ntraj, bb, origin, &t, &b);
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)a.Cc, a.C - c0);
    __syncthreads();
    load_patch<R, D>(geo, grid, b * a.C + c0, a.gtot, ncl, a.cells, a.ps, origin, patch);
    __syncthreads();
    const int nrounds = (it.len + ppb - 1) / ppb;
    for (int r = 0; r < nrounds; ++r) {
      const int s = r * ppb + warp * ppw + lane / a.Cc;
      const bool active = s < it.len;
      const int64_t i = it.start + (active ? s : 0);
      R om[D], tm[D];
      int base[D], local[D];
      bool ok = active;
      cplx<R> hv[D][kMaxJ], hd[D][kMaxJ];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        om[d] = coords[d * a.n + i];
        ok &= base_index<R>(om[d], geo.gam[d], geo.halfJ[d], &tm[d], &base[d]);
        local[d] = pmod(base[d], geo.K[d]) - origin[d];
        ok &= (local[d] >= 0) & (local[d] < geo.T[d]);
#pragma unroll
        for (int j = 0; j < kMaxJ; ++j) {
          if (j < geo.J[d]) {
            lerp_tables<R>(geo, d, tm[d], base[d] + j, &hv[d][j], &hd[d][j]);
          } else {
            hv[d][j] = mk<R>(0, 0);
            hd[d][j] = mk<R>(0, 0);
          }
        }
      }
      R gsum[D];
#pragma unroll
      for (int d = 0; d < D; ++d) gsum[d] = R(0);
      int64_t m = 0;
      if (ok) m = a.vals[i] - t * a.M;
      if (ok && c < ncl) {
        const cplx<R>* plane = patch + c * a.ps;
        // value and per-dim derivative sums
        cplx<R> val = mk<R>(0, 0);
        cplx<R> der[D];
#pragma unroll
        for (int d = 0; d < D; ++d) der[d] = mk<R>(0, 0);
        if (D == 1) {
          for (int j = 0; j < geo.J[0]; ++j) {
            const cplx<R> x = plane[local[0] + j];
            val = cfma<R>(hv[0][j], x, val);
            der[0] = cfma<R>(hd[0][j], x, der[0]);
          }
        } else if (D == 2) {
          for (int jy = 0; jy < geo.J[0]; ++jy) {
            cplx<R> rv = mk<R>(0, 0), rd = mk<R>(0, 0);
            const cplx<R>* row = plane + (local[0] + jy) * geo.P[1 % D] + local[1 % D];
#pragma unroll
            for (int jx = 0; jx < kMaxJ; ++jx) {
              if (jx < geo.J[1 % D]) {
                const cplx<R> x = row[jx];
                rv = cfma<R>(hv[1 % D][jx], x, rv);
                rd = cfma<R>(hd[1 % D][jx], x, rd);
              }
            }
            val = cfma<R>(hv[0][jy], rv, val);
            der[0] = cfma<R>(hd[0][jy], rv, der[0]);
            der[1 % D] = cfma<R>(hv[0][jy], rd, der[1 % D]);
          }
        } else {
          for (int jz = 0; jz < geo.J[0]; ++jz) {
            cplx<R> zv = mk<R>(0, 0), zdy = mk<R>(0, 0), zdx = mk<R>(0, 0);
            for (int jy = 0; jy < geo.J[1 % D]; ++jy) {
              cplx<R> rv = mk<R>(0, 0), rd = mk<R>(0, 0);
              const cplx<R>* row =
                  plane + ((local[0] + jz) * geo.P[1 % D] + local[1 % D] + jy) * geo.P[2 % D] + local[2 % D];
#pragma unroll
              for (int jx = 0; jx < kMaxJ; ++jx) {
                if (jx < geo.J[2 % D]) {
                  const cplx<R> x = row[jx];
                  rv = cfma<R>(hv[2 % D][jx], x, rv);
                  rd = cfma<R>(hd[2 % D][jx], x, rd);
                }
              }
              zv = cfma<R>(hv[1 % D][jy], rv, zv);
              zdy = cfma<R>(hd[1 % D][jy], rv, zdy);
              zdx = cfma<R>(hv[1 % D][jy], rd, zdx);
            }
            val = cfma<R>(hv[0][jz], zv, val);
            der[0] = cfma<R>(hd[0][jz], zv, der[0]);
            der[1 % D] = cfma<R>(hv[0][jz], zdy, der[1 % D]);
            der[2 % D] = cfma<R>(hv[0][jz], zdx, der[2 % D]);
          }
        }
        R sn, cs;
        sincos_acc(phase_arg<R, D>(om, geo.nshift), &sn, &cs);
        const cplx<R> ph = mk<R>(cs, sn);
        const cplx<R> vv = v[(b * a.C + c0 + c) * a.M + m];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          // dy/d omega_d = phase * (der_d / gam_d + i * nshift_d * val)
          const cplx<R> inner = mk<R>(der[d].x / geo.gam[d] - geo.nshift[d] * val.y,
                                      der[d].y / geo.gam[d] + geo.nshift[d] * val.x);
          const cplx<R> dy = cmul<R>(ph, inner);
          gsum[d] = vv.x * dy.x + vv.y * dy.y;  // Re(conj(v) * dy)
        }
      }
      // reduce over the Cc lanes of this point (lanes of one point are contiguous)
#pragma unroll
      for (int d = 0; d < D; ++d) {
        for (int off = a.Cc >> 1; off > 0; off >>= 1) gsum[d] += __shfl_down_sync(0xffffffffu, gsum[d], off, a.Cc);
      }
      if (ok && c == 0) {
#pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(&grad[(t * D + d) * a.M + m], gsum[d]);
      }
      if (active && !ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
  }
}

}  // namespace tkbn

namespace tkbn_host {

using namespace tkbn;

static int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

struct InterpPlan {
  PointsLayout L;
  Launch a;
  size_t smem;
  int64_t max_jobs;
};

template <typename R>
static int prepare(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, int64_t B, int64_t C,
                   InterpPlan* ip) {
  int rc = points_layout(g, p, &ip->L);
  if (rc) return rc;
  if (!ws) return set_error(TKBN_ERR_INVALID, "points workspace is null");
  if (B < 1 || C < 1) return set_error(TKBN_ERR_INVALID, "batch and coil counts must be >= 1");
  if (p->ntraj != 1 && p->ntraj != B)
    return set_error(TKBN_ERR_INVALID, "If omega has batch dim, omega batch dimension must match image.");
  for (int d = 0; d < g->ndim; ++d) {
    if (g->numpoints[d] < 1 || g->numpoints[d] > kMaxJ)
      return set_error(TKBN_ERR_UNSUPPORTED, "numpoints must be in [1, %d]", kMaxJ);
    if (g->table_oversamp[d] < 1) return set_error(TKBN_ERR_INVALID, "table_oversamp must be >= 1");
  }
  const char* base = (const char*)ws;
  Launch& a = ip->a;
  a.items = (const Item*)(base + ip->L.off_items);
  a.hdr = (const int64_t*)(base + ip->L.off_hdr);
  a.vals = (const int32_t*)(base + ip->L.off_vals);
  a.n = ip->L.npts_total;
  a.M = p->npts;
  a.ntraj = p->ntraj;
  a.B = B;
  a.C = C;
  // coil chunk: power of two, <= 16 (<= 8 for complex128), covering C when possible
  const int cmax = g->dtype == TKBN_C64 ? 16 : 8;
  a.Cc = next_pow2((int)(C < cmax ? C : cmax));
  a.ncc = (int)((C + a.Cc - 1) / a.Cc);
  a.nbpt = p->ntraj == 1 ? B : 1;
  int cells = 1;
  a.gtot = 1;
  for (int d = 0; d < g->ndim; ++d) {
    cells *= ip->L.tile[d] + g->numpoints[d] - 1;
    a.gtot *= g->grid_size[d];
  }
  a.cells = cells;
  a.ps = cells | 1;  // odd plane stride spreads coil planes over banks
  ip->smem = (size_t)a.Cc * a.ps * sizeof(cplx<R>);
  if (ip->smem > 220 * 1024)
    return set_error(TKBN_ERR_UNSUPPORTED, "tile patch needs %zu bytes of shared memory", ip->smem);
  ip->max_jobs = ip->L.max_items * a.nbpt * a.ncc;
  return TKBN_OK;
}

// Persistent grid: as many CTAs as are resident at once (no second wave), at
// most one per job.
template <typename K>
static int resident_blocks(K kernel, size_t smem, int64_t max_jobs, int* blocks) {
  int rc = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "smem attribute");
  if (rc) return rc;
  int dev = 0, sms = 0, per_sm = 0;
  if ((rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
  if ((rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))) return rc;
  if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem), "occupancy")))
    return rc;
  if (per_sm < 1) return set_error(TKBN_ERR_UNSUPPORTED, "interpolation kernel cannot be resident with %zu B smem", smem);
  int64_t b = (int64_t)per_sm * sms;
  if (max_jobs < b) b = max_jobs;
  *blocks = (int)(b < 1 ? 1 : b);
  return TKBN_OK;
}

template <typename R, int D, int JC>
static int launch_fwd_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* grid, void* kdata,
                        cudaStream_t s) {
  auto k = k_interp_fwd<R, D, JC>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords), (const cplx<R>*)grid,
                                         (cplx<R>*)kdata);
  return check_cuda(cudaGetLastError(), "interp_fwd launch");
}

template <typename R, int D, int JC>
static int launch_adj_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* kdata, void* grid,
                        cudaStream_t s) {
  auto k = k_interp_adj<R, D, JC>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords), (const cplx<R>*)kdata,
                                         (cplx<R>*)grid);
  return check_cuda(cudaGetLastError(), "interp_adj launch");
}

static bool all_j(const tkbn_geometry* g, int j) {
  for (int d = 0; d < g->ndim; ++d)
    if (g->numpoints[d] != j) return false;
  return true;
}

template <typename R>
static int interp_fwd_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                        const void* grid, int64_t B, int64_t C, void* kdata, cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, &ip);
  if (rc) return rc;
  if (p->npts == 0) return TKBN_OK;
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, nullptr);
  const char* w = (const char*)ws;
  const bool j6 = all_j(g, 6);
  switch (g->ndim) {
    case 1:
      return j6 ? launch_fwd_t<R, 1, 6>(geo, ip, w, grid, kdata, s) : launch_fwd_t<R, 1, 0>(geo, ip, w, grid, kdata, s);
    case 2:
      return j6 ? launch_fwd_t<R, 2, 6>(geo, ip, w, grid, kdata, s) : launch_fwd_t<R, 2, 0>(geo, ip, w, grid, kdata, s);
    default:
      return j6 ? launch_fwd_t<R, 3, 6>(geo, ip, w, grid, kdata, s) : launch_fwd_t<R, 3, 0>(geo, ip, w, grid, kdata, s);
  }
}

template <typename R>
static int interp_adj_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                        const void* kdata, int64_t B, int64_t C, void* grid, cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, &ip);
  if (rc) return rc;
  rc = check_cuda(cudaMemsetAsync(grid, 0, (size_t)(B * C * ip.a.gtot) * sizeof(cplx<R>), s), "zero grid");
  if (rc || p->npts == 0) return rc;
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, nullptr);
  const char* w = (const char*)ws;
  const bool j6 = all_j(g, 6);
  switch (g->ndim) {
    case 1:
      return j6 ? launch_adj_t<R, 1, 6>(geo, ip, w, kdata, grid, s) : launch_adj_t<R, 1, 0>(geo, ip, w, kdata, grid, s);
    case 2:
      return j6 ? launch_adj_t<R, 2, 6>(geo, ip, w, kdata, grid, s) : launch_adj_t<R, 2, 0>(geo, ip, w, kdata, grid, s);
    default:
      return j6 ? launch_adj_t<R, 3, 6>(geo, ip, w, kdata, grid, s) : launch_adj_t<R, 3, 0>(geo, ip, w, kdata, grid, s);
  }
}

template <typename R, int D>
static int launch_grad_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* grid, const void* v,
                         void* grad, cudaStream_t s) {
  auto k = k_interp_grad<R, D>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords), (const cplx<R>*)grid,
                                         (const cplx<R>*)v, (R*)grad);
  return check_cuda(cudaGetLastError(), "interp_grad launch");
}

template <typename R>
static int interp_grad_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                         const void* const* dtables, const void* grid, const void* v, int64_t B, int64_t C,
                         void* grad, cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, &ip);
  if (rc) return rc;
  if (!dtables) return set_error(TKBN_ERR_INVALID, "derivative tables are required");
  rc = check_cuda(cudaMemsetAsync(grad, 0, (size_t)(p->ntraj * g->ndim * p->npts) * sizeof(R), s), "zero grad");
  if (rc || p->npts == 0) return rc;
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, dtables);
  const char* w = (const char*)ws;
  switch (g->ndim) {
    case 1:
      return launch_grad_t<R, 1>(geo, ip, w, grid, v, grad, s);
    case 2:
      return launch_grad_t<R, 2>(geo, ip, w, grid, v, grad, s);
    default:
      return launch_grad_t<R, 3>(geo, ip, w, grid, v, grad, s);
  }
}

int interp_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
               const void* grid, int64_t B, int64_t C, void* kdata, cudaStream_t s) {
  if (g->dtype == TKBN_C64) return interp_fwd_r<float>(g, p, ws, tables, grid, B, C, kdata, s);
  if (g->dtype == TKBN_C128) return interp_fwd_r<double>(g, p, ws, tables, grid, B, C, kdata, s);
  return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", g->dtype);
}

int interp_adj(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
               const void* kdata, int64_t B, int64_t C, void* grid, cudaStream_t s) {
  if (g->dtype == TKBN_C64) return interp_adj_r<float>(g, p, ws, tables, kdata, B, C, grid, s);
  if (g->dtype == TKBN_C128) return interp_adj_r<double>(g, p, ws, tables, kdata, B, C, grid, s);
  return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", g->dtype);
}

int interp_grad(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                const void* const* dtables, const void* grid, const void* v, int64_t B, int64_t C, void* grad,
                cudaStream_t s) {
  if (g->dtype == TKBN_C64) return interp_grad_r<float>(g, p, ws, tables, dtables, grid, v, B, C, grad, s);
  if (g->dtype == TKBN_C128) return interp_grad_r<double>(g, p, ws, tables, dtables, grid, v, B, C, grad, s);
  return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", g->dtype);
}

}  // namespace tkbn_host

TKBN_DEFINE_STATUS_READER(status_interp)
