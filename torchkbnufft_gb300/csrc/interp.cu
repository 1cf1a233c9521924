// K3 (gather), K4 (scatter) and K7 (trajectory-gradient gather) on the
// bin-sorted layout.
//
// One work item = up to `chunk` points whose footprints start inside one grid
// tile. A CTA takes a job (item, batch, coil chunk), stages the tile's patch
// (tile + J-1 halo, wrapped periodically) of Cc coil planes in shared memory,
// and processes the item's points with Cc lanes per point (lane = coil).
// The J^d table coefficients of a point are computed once per point: its Cc
// lanes each evaluate some of the D*J per-dimension table factors and share
// them through a per-warp shared-memory scratch. The normalised frequency tm
// and the fftshift phase of every point come precomputed from the layout.
//
// Reference semantics (mmuckley/torchkbnufft):
//   forward  y[b,c,m] = phase_m * sum_j coef_j(m) * X[b,c,idx_j(m)]
//            (table_interp_one_batch, torchkbnufft/_nufft/interp.py:153-203)
//   adjoint  X[b,c,idx_j(m)] += conj(coef_j(m)) * conj(phase_m) * y[b,c,m]
//            (table_interp_adjoint, torchkbnufft/_nufft/interp.py:587-726)
// The separable sums group the products per dimension; the table bins, cell
// indices and phase argument are computed exactly as the reference does.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "geo_host.cuh"
#include "tkbn_common.cuh"

namespace tkbn {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

template <int JC>
struct NJOf {
  static constexpr int N = JC > 0 ? JC : kMaxJ;
};

struct Launch {
  const Item* items;
  const int64_t* hdr;   // hdr[0] = number of items
  const int32_t* vals;  // sorted -> original flat index t*M + m
  int64_t n;            // ntraj * M
  int64_t M;
  int64_t ntraj;
  int64_t B, C;
  int Cc;               // coils per job (power of two <= 32)
  int ncc;              // coil chunks
  int64_t nbpt;         // batch items per trajectory job (B if shared trajectory else 1)
  int cells;            // prod P
  int ps;               // smem plane stride (elements)
  int64_t gtot;         // prod K
  int scratch;          // per-warp factor scratch (complex elements)
};

template <typename R>
__device__ __forceinline__ void job_decode(const Geo<R>& geo, const Item& it, int64_t ntraj, int64_t bb, int* origin,
                                           int64_t* t_out, int64_t* b_out) {
  const int64_t t = it.key / geo.ntiles;
  int rem = (int)(it.key - t * geo.ntiles);
#pragma unroll
  for (int d = kMaxDim - 1; d >= 0; --d) {
    if (d < geo.ndim) {
      const int td = rem % geo.ntile[d];
      rem /= geo.ntile[d];
      origin[d] = td * geo.T[d];
    } else {
      origin[d] = 0;
    }
  }
  *t_out = t;
  *b_out = ntraj == 1 ? bb : t;
}

// Per-point data every lane needs: tm, the first footprint cell and its
// offset inside the tile patch. False for a non-finite point or a point whose
// footprint does not start inside this tile.
template <typename R, int D>
__device__ __forceinline__ bool point_base(const Geo<R>& geo, const R* __restrict__ tm, int64_t n, int64_t i,
                                           const int* origin, R* tmv, int* base, int* local) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const R t = tm[d * n + i];
    tmv[d] = t;
    const R f = floor(sub_rn(t, geo.halfJ[d]));
    const bool fin = fabs(f) < R(1 << 30);
    base[d] = fin ? 1 + (int)f : 0;
    const int l = wrap_cell(base[d], geo.K[d]) - origin[d];
    local[d] = l;
    ok = ok && fin && (l >= 0) && (l < geo.T[d]);
  }
  return ok;
}

// point_base with tm already in registers.
template <typename R, int D>
__device__ __forceinline__ bool point_base_at(const Geo<R>& geo, const R* tmv, const int* origin, int* base,
                                              int* local) {
  bool ok = true;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const R f = floor(sub_rn(tmv[d], geo.halfJ[d]));
    const bool fin = fabs(f) < R(1 << 30);
    base[d] = fin ? 1 + (int)f : 0;
    const int l = wrap_cell(base[d], geo.K[d]) - origin[d];
    local[d] = l;
    ok = ok && fin && (l >= 0) && (l < geo.T[d]);
  }
  return ok;
}

template <typename T, int D>
__device__ __forceinline__ T sel(const T* v, int d) {
  return (D > 2 && d == 2) ? v[2 % D] : ((D > 1 && d == 1) ? v[1 % D] : v[0]);
}

// Table factors h[d][j] = table_d[bin(tm_d, base_d + j)]. With coop, the
// `lanes` lanes of a point split the D*NJ evaluations and exchange them via
// `scr` (per-point scratch); every lane of the warp must call this.
template <typename R, int D, int JC>
__device__ __forceinline__ void table_factors(const Geo<R>& geo, const R* tmv, const int* base, int lane_in_pt,
                                              int lanes, bool coop, cplx<R>* scr, cplx<R> (&h)[D][NJOf<JC>::N]) {
  constexpr int NJ = NJOf<JC>::N;
  if (coop) {
    for (int f = lane_in_pt; f < D * NJ; f += lanes) {
      const int d = f / NJ, j = f - (f / NJ) * NJ;
      const int J = JC > 0 ? JC : sel<int, 3>(geo.J, d);
      cplx<R> v = mk<R>(0, 0);
      if (j < J) {
        const int k = table_bin<R>(sel<R, D>(tmv, d), sel<int, D>(base, d) + j, sel<R, 3>(geo.Lr, d),
                                   sel<int, 3>(geo.center, d), sel<int, 3>(geo.tmax, d));
        v = table_entry<R>(sel<const cplx<R>*, 3>(geo.tab, d), k, sel<int, 3>(geo.center, d), sel<bool, 3>(geo.half, d));
      }
      scr[f] = v;
    }
    __syncwarp();
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int j = 0; j < NJ; ++j) h[d][j] = scr[d * NJ + j];
    __syncwarp();
  } else {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int J = JC > 0 ? JC : geo.J[d];
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        h[d][j] = mk<R>(0, 0);
        if (j < J)
          h[d][j] = table_entry<R>(geo.tab[d], table_bin<R>(tmv[d], base[d] + j, geo.Lr[d], geo.center[d], geo.tmax[d]),
                                   geo.center[d], geo.half[d]);
      }
    }
  }
}

// Non-negative x reduced into [0, k) by repeated subtraction (patch offsets
// exceed k by less than one tile, so this is one compare in practice).
__device__ __forceinline__ int wrap_up(int x, int k) {
  while (x >= k) x -= k;
  return x;
}

// Global offset of patch row rr (the outer coordinates of a row of P[D-1]
// cells), wrapped periodically.
template <typename R, int D>
__device__ __forceinline__ int64_t patch_row_base(const Geo<R>& geo, int rr, const int* origin) {
  if (D == 1) return 0;
  if (D == 2) return (int64_t)wrap_up(origin[0] + rr, geo.K[0]) * geo.K[1];
  const int pz = rr / geo.P[1 % D];
  const int py = rr - pz * geo.P[1 % D];
  return ((int64_t)wrap_up(origin[0] + pz, geo.K[0]) * geo.K[1 % D] + wrap_up(origin[1 % D] + py, geo.K[1 % D])) *
         geo.K[2 % D];
}

// Stage Cc coil planes of the periodic patch [origin, origin + P) into smem:
// one warp per patch row, lanes along the innermost dimension; each lane
// wraps its column offsets once per job.
// Asynchronous global -> shared copy of one complex element (cp.async,
// cached in L1): a thread issues all of its patch copies back to back and
// waits once, instead of one load latency per element.
__device__ __forceinline__ void cp_async_elem(float2* smem_dst, const float2* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_elem(double2* smem_dst, const double2* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_16(float2* smem_dst, const float2* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Tensor-memory-access store of a 3D box from shared memory (bulk group).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* smem, int x, int y, int z) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];\n" ::"l"(map),
               "r"(s), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

template <typename R, int D>
__device__ __forceinline__ void load_patch(const Geo<R>& geo, const cplx<R>* __restrict__ grid, int64_t plane0,
                                           int64_t gtot, int ncl, int cells, int ps, const int* origin,
                                           cplx<R>* patch) {
  const int PX = geo.P[D - 1];
  const int KX = geo.K[D - 1];
  const int rows = cells / PX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (PX <= 16) {
    // short rows (3D tiles): each half-warp copies one row
    const int half = lane >> 4, hl = lane & 15;
    const int gx = wrap_up(origin[D - 1] + hl, KX);
    for (int rr = 2 * warp + half; rr < rows; rr += 2 * kWarps) {
      const int64_t rbase = patch_row_base<R, D>(geo, rr, origin);
      if (hl < PX)
        for (int c = 0; c < ncl; ++c) cp_async_elem(patch + c * ps + rr * PX + hl, grid + (plane0 + c) * gtot + rbase + gx);
    }
  } else {
    const int gx0 = wrap_up(origin[D - 1] + lane, KX);
    for (int rr = warp; rr < rows; rr += kWarps) {
      const int64_t rbase = patch_row_base<R, D>(geo, rr, origin);
      for (int c = 0; c < ncl; ++c) {
        const cplx<R>* src = grid + (plane0 + c) * gtot + rbase;
        cplx<R>* dst = patch + c * ps + rr * PX;
        int gx = gx0;
        for (int px = lane; px < PX; px += 32) {
          cp_async_elem(dst + px, src + gx);
          gx = wrap_up(gx + 32, KX);
        }
      }
    }
  }
  // every copy of this thread has landed; the caller's barrier publishes them
  cp_async_wait_all();
}

// f[j] for a runtime j through a select chain: indexing the register array
// directly would move the whole factor array to local memory.
template <typename R, int NJ>
__device__ __forceinline__ cplx<R> pick_factor(const cplx<R> (&f)[NJ], int j) {
  cplx<R> v = f[0];
#pragma unroll
  for (int q = 1; q < NJ; ++q)
    if (q == j) v = f[q];
  return v;
}

template <typename R, int D, int JC>
__device__ __forceinline__ cplx<R> gather_point(const Geo<R>& geo, const cplx<R> (&h)[D][NJOf<JC>::N],
                                                const int* local, const cplx<R>* __restrict__ plane) {
  constexpr int NJ = NJOf<JC>::N;
  cplx<R> acc = mk<R>(0, 0);
  if (D == 1) {
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (JC > 0 || j < geo.J[0]) acc = cfma<R>(h[0][j], plane[local[0] + j], acc);
  } else if (D == 2) {
    const int P1 = geo.P[1];
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      if (JC > 0 || jy < geo.J[0]) {
        const cplx<R>* row = plane + (local[0] + jy) * P1 + local[1 % D];
        cplx<R> r = mk<R>(0, 0);
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx)
          if (JC > 0 || jx < geo.J[1 % D]) r = cfma<R>(h[1 % D][jx], row[jx], r);
        acc = cfma<R>(h[0][jy], r, acc);
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
            const cplx<R>* row = plane + ((local[0] + jz) * P1 + local[1 % D] + jy) * P2 + local[2 % D];
            cplx<R> r = mk<R>(0, 0);
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx)
              if (JC > 0 || jx < geo.J[2 % D]) r = cfma<R>(h[2 % D][jx], row[jx], r);
            sz = cfma<R>(h[1 % D][jy], r, sz);
          }
        }
        acc = cfma<R>(pick_factor<R, NJ>(h[0], jz), sz, acc);
      }
    }
  }
  return acc;
}

// Global-memory flush: one vector atomic for float2 (sm_90+), two for double.
__device__ __forceinline__ void atomic_add_global(float2* p, float2 v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_global(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// Adjoint accumulation planes: real and imaginary parts in separate planes
// (re plane c at c*ps, im plane c at (Cc + c)*ps), so that the Cc lanes of a
// point hit Cc distinct banks with an odd plane stride.
template <typename R, int D, int JC>
__device__ __forceinline__ void scatter_point(const Geo<R>& geo, const cplx<R> (&h)[D][NJOf<JC>::N],
                                              const int* local, cplx<R> v, R* pre, R* pim) {
  constexpr int NJ = NJOf<JC>::N;
  if (D == 1) {
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      if (JC > 0 || j < geo.J[0]) {
        const cplx<R> w = cmulc<R>(v, h[0][j]);
        atomicAdd(&pre[local[0] + j], w.x);
        atomicAdd(&pim[local[0] + j], w.y);
      }
    }
  } else if (D == 2) {
    const int P1 = geo.P[1];
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      if (JC > 0 || jy < geo.J[0]) {
        const cplx<R> vy = cmulc<R>(v, h[0][jy]);
        const int row = (local[0] + jy) * P1 + local[1 % D];
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx) {
          if (JC > 0 || jx < geo.J[1 % D]) {
            const cplx<R> w = cmulc<R>(vy, h[1 % D][jx]);
            atomicAdd(&pre[row + jx], w.x);
            atomicAdd(&pim[row + jx], w.y);
          }
        }
      }
    }
  } else {
    const int P1 = geo.P[1 % D], P2 = geo.P[2 % D];
#pragma unroll 1
    for (int jz = 0; jz < NJ; ++jz) {
      if (JC > 0 || jz < geo.J[0]) {
        const cplx<R> vz = cmulc<R>(v, pick_factor<R, NJ>(h[0], jz));
#pragma unroll
        for (int jy = 0; jy < NJ; ++jy) {
          if (JC > 0 || jy < geo.J[1 % D]) {
            const cplx<R> vy = cmulc<R>(vz, h[1 % D][jy]);
            const int row = ((local[0] + jz) * P1 + local[1 % D] + jy) * P2 + local[2 % D];
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx) {
              if (JC > 0 || jx < geo.J[2 % D]) {
                const cplx<R> w = cmulc<R>(vy, h[2 % D][jx]);
                atomicAdd(&pre[row + jx], w.x);
                atomicAdd(&pim[row + jx], w.y);
              }
            }
          }
        }
      }
    }
  }
}

template <typename R, int D>
__device__ __forceinline__ void flush_patch(const Geo<R>& geo, cplx<R>* __restrict__ grid, int64_t plane0,
                                            int64_t gtot, int ncl, int cells, int ps, int Cc, const int* origin,
                                            const R* pre, const R* pim) {
  const int PX = geo.P[D - 1];
  const int KX = geo.K[D - 1];
  const int rows_per_plane = cells / PX;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = warp; r < ncl * rows_per_plane; r += kWarps) {
    const int c = r / rows_per_plane;
    const int rr = r - c * rows_per_plane;
    cplx<R>* dst = grid + (plane0 + c) * gtot + patch_row_base<R, D>(geo, rr, origin);
    // pre and pim are the bases of the real and imaginary plane sets
    const int o = c * ps + rr * PX;
    for (int px = lane; px < PX; px += 32) {
      const cplx<R> v = mk<R>(pre[o + px], pim[o + px]);
      if (v.x == R(0) && v.y == R(0)) continue;
      int gx = origin[D - 1] + px;
      gx = gx >= KX ? gx - KX * (gx / KX) : gx;
      atomic_add_global(&dst[gx], v);
    }
  }
}

// Common job loop skeleton pieces ------------------------------------------

struct JobCtx {
  int64_t t, b;
  int c0, ncl;
  int origin[kMaxDim];
};

template <typename R>
__device__ __forceinline__ bool next_job(const Geo<R>& geo, const Launch& a, int64_t job, int64_t nitems, Item* it,
                                         JobCtx* j) {
  const int64_t item_idx = job % nitems;
  const int64_t rest = job / nitems;
  const int cc = (int)(rest % a.ncc);
  const int64_t bb = rest / a.ncc;
  *it = a.items[item_idx];
  job_decode<R>(geo, *it, a.ntraj, bb, j->origin, &j->t, &j->b);
  j->c0 = cc * a.Cc;
  j->ncl = (int)min((int64_t)a.Cc, a.C - j->c0);
  return true;
}

// One gather job (a work item of one batch item and coil chunk). All
// threads of the CTA call it; `patch` is the dynamic shared memory.
template <typename R, int D, int JC>
__device__ __forceinline__ void fwd_job(const Geo<R>& geo, const Launch& a, const R* __restrict__ tm,
                                        const cplx<R>* __restrict__ ph, const cplx<R>* __restrict__ grid,
                                        cplx<R>* __restrict__ kdata, int64_t job, int64_t nitems, cplx<R>* patch) {
  constexpr int NJ = NJOf<JC>::N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  cplx<R>* scr_warp = patch + a.Cc * a.ps + warp * a.scratch;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * kWarps;
  const int c = lane % a.Cc;
  const int pslot = lane / a.Cc;
  const bool coop = a.Cc >= 4;
  cplx<R>* scr = scr_warp + pslot * (D * NJ);
  {
    Item it;
    JobCtx jc;
    next_job<R>(geo, a, job, nitems, &it, &jc);
    __syncthreads();
    load_patch<R, D>(geo, grid, jc.b * a.C + jc.c0, a.gtot, jc.ncl, a.cells, a.ps, jc.origin, patch);
    __syncthreads();
    const int nrounds = (it.len + ppb - 1) / ppb;
    // the next round's point data is loaded one round ahead (hides its latency)
    int64_t i_next = it.start + min(warp * ppw + pslot, it.len - 1);
    R tm_next[D];
    int32_t val_next = a.vals[i_next];
    cplx<R> ph_next = ph[i_next];
#pragma unroll
    for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
    for (int r = 0; r < nrounds; ++r) {
      const int s = r * ppb + warp * ppw + pslot;
      const bool active = s < it.len;
      R tmv[D];
#pragma unroll
      for (int d = 0; d < D; ++d) tmv[d] = tm_next[d];
      const int32_t val = val_next;
      const cplx<R> phv = ph_next;
      if (r + 1 < nrounds) {
        i_next = it.start + min(s + ppb, it.len - 1);
        val_next = a.vals[i_next];
        ph_next = ph[i_next];
#pragma unroll
        for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
      }
      int base[D], local[D];
      const bool ok = point_base_at<R, D>(geo, tmv, jc.origin, base, local);
      cplx<R> h[D][NJ];
      table_factors<R, D, JC>(geo, tmv, base, c, a.Cc, coop, scr, h);
      if (active && c < jc.ncl) {
        const int64_t m = val - jc.t * a.M;
        cplx<R> y;
        if (ok) {
          y = cmul<R>(gather_point<R, D, JC>(geo, h, local, patch + c * a.ps), phv);
        } else {
          y = mk<R>(R(NAN), R(NAN));
        }
        kdata[(jc.b * a.C + jc.c0 + c) * a.M + m] = y;
      }
      if (active && !ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
  }
}

// 2D register-adjoint tile (rows x columns) and coils per job; the
// linear-phase gather and adjoint below share its E tables.
constexpr int kRegTileY = 16, kRegTileX = 14, kRegCoils = 16;

// Linear-phase tables (TKBN_TABLES_LINEAR_PHASE): table[k] = m(k) e^{i c u_k},
// u_k = (k - center) / L, m >= 0. A point's factors sit at u_0 - j (u_0 in
// (J/2 - 1, J/2]), so with E[n] = e^{-i c n} and h^ = h / |h|,
//   e^{-i c u_0} = conj(h^[2]) E[2]       (h[2]: |u| <= 1, a well-defined phase)
// and, with tile-local cell (y, x) and footprint start (ry, rx), jy = y - ry:
//   conj(hy[jy] hx[jx] phase) = my[jy] mx[jx] * Q * R(y, x),
//   Q = conj(phase hy^[2] hx^[2]) Ey[2 + ry] Ex[2 + rx],  R(y, x) = conj(Ey[y] Ex[x]).
// The adjoint multiplies the k-space values by Q (per list entry),
// accumulates with the real my, mx and multiplies the tile by R. The slope c
// is fitted by least squares to the table's phases over u in (0, 1] (error
// ~1e-8), and the E tables are evaluated in double.
constexpr int kLpE0 = 3;              // E tables start at n = -kLpE0
constexpr int kLpEy = kRegTileY + 5;  // n = -3 .. 17 (entries 2 + ry and cells y)
constexpr int kLpEx = kRegTileX + 5;  // n = -3 .. 15

// ---------------------------------------------------------------- K3, coil pairs
// Gather for 2D complex64, J = 6, CC coils per job (2, 4, 8 or 16): the tile
// patch is stored coil-fastest ([cell][CC + 2]), so a lane reads two coils of a
// cell with one 16-byte load and the point's per-lane work (coordinates,
// table factors, addressing) is shared by two coils. Lanes are (point slot,
// coil pair): 64 / CC points per warp.
// Coil-pair patch cell: CC coils then 16 unused bytes, so that lanes copying
// consecutive columns of one coil write to different banks while the lanes
// of a point still read one cell's CC coils as contiguous 16-byte pairs.
template <int CC>
__host__ __device__ constexpr int pair_cell_stride() {
  return CC + 2;
}

template <int CC>
__device__ __forceinline__ void load_patch_pairs(const Geo<float>& geo, const float2* __restrict__ grid,
                                                 int64_t plane0, int64_t gtot, int ncl, const int* origin,
                                                 float2* patch) {
  constexpr int CS = pair_cell_stride<CC>();
  const int PX = geo.P[1], PY = geo.P[0], KX = geo.K[1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int rr = warp; rr < PY; rr += kWarps) {
    const int64_t rbase = patch_row_base<float, 2>(geo, rr, origin);
    for (int x = lane; x < PX; x += 32) {
      const float2* src = grid + plane0 * gtot + rbase + wrap_cell(origin[1] + x, KX);
      float2* dst = patch + (rr * PX + x) * CS;
#pragma unroll 4
      for (int c = 0; c < CC; ++c) {
        if (c < ncl)
          cp_async_elem(dst + c, src + c * gtot);
        else
          dst[c] = make_float2(0.f, 0.f);
      }
    }
  }
  cp_async_wait_all();
}

// LP (linear-phase tables, see kLpE0): real kernel values from the per-point
// pre-pass records {mx[6], my[6], P} (P = conj(phase hy^[2] hx^[2])). Patch
// cell (Y, X) is multiplied once per job by Ey[Y - 3] Ex[X - 3], so that with
// the footprint start (ly, lx) in the patch and Y = ly + jy, E[jy - 2] =
// E[Y - 3] conj(E[ly - 1]) gives
//   y = conj(P Ey[ly - 1] Ex[lx - 1]) sum_jy my[jy] sum_jx mx[jx] X'(ly + jy, lx + jx):
// two real multiply-adds per tap and coil instead of four. Points whose bins
// do not step by exactly L have P = 0 here and are rewritten by k_fwd_lp_fix.
// pfr: the records (16 floats per sorted point); etab: {Ey[kLpEy], Ex[kLpEx]}
// in shared memory; the patch must be at most kLpEy x kLpEx cells.
template <int CC, bool LP = false>
__device__ __forceinline__ void fwd_job_pairs(const Geo<float>& geo, const Launch& a, const float* __restrict__ tm,
                                              const float2* __restrict__ ph, const float2* __restrict__ grid,
                                              float2* __restrict__ kdata, int64_t job, int64_t nitems,
                                              float2* patch, const float* __restrict__ pfr = nullptr,
                                              const float2* etab = nullptr) {
  constexpr int D = 2, NJ = 6, LPP = CC / 2, PPW = 32 / LPP;  // lanes per point, points per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int PX = geo.P[1];
  const int cells = geo.P[0] * PX;
  constexpr int CS = pair_cell_stride<CC>();
  float2* scr = patch + cells * CS + warp * (PPW * D * NJ);
  const int k = lane % LPP;       // coil pair: coils 2k, 2k+1 of the chunk
  const int pslot = lane / LPP;   // point slot in the warp
  float2* pscr = scr + pslot * (D * NJ);
  Item it;
  JobCtx jc;
  next_job<float>(geo, a, job, nitems, &it, &jc);
  __syncthreads();
  load_patch_pairs<CC>(geo, grid, jc.b * a.C + jc.c0, a.gtot, jc.ncl, jc.origin, patch);
  __syncthreads();
  if constexpr (LP) {
    // the patch times Ey[Y - 3] Ex[X - 3] (thread per cell, 16 bytes at a time)
    for (int cell = threadIdx.x; cell < cells; cell += kThreads) {
      const int Y = cell / PX, X = cell - Y * PX;
      const float2 E = cmul<float>(etab[Y], etab[kLpEy + X]);
      float4* pc = reinterpret_cast<float4*>(patch + cell * CS);
#pragma unroll
      for (int q = 0; q < CC / 2; ++q) {
        const float4 v = pc[q];
        const float2 v0 = cmul<float>(make_float2(v.x, v.y), E), v1 = cmul<float>(make_float2(v.z, v.w), E);
        pc[q] = make_float4(v0.x, v0.y, v1.x, v1.y);
      }
    }
    __syncthreads();
  }
  constexpr int PPB = PPW * kWarps;
  const int nrounds = (it.len + PPB - 1) / PPB;
  int64_t i_next = it.start + min(warp * PPW + pslot, it.len - 1);
  float tm_next[D];
  int32_t val_next = a.vals[i_next];
  float2 ph_next = make_float2(0.f, 0.f);
  float4 rec_next[4];
  if constexpr (LP) {
#pragma unroll
    for (int q = 0; q < 4; ++q) rec_next[q] = reinterpret_cast<const float4*>(pfr + i_next * 16)[q];
  } else {
    ph_next = ph[i_next];
  }
#pragma unroll
  for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
  for (int r = 0; r < nrounds; ++r) {
    const int s = r * PPB + warp * PPW + pslot;
    const bool active = s < it.len;
    float tmv[D];
#pragma unroll
    for (int d = 0; d < D; ++d) tmv[d] = tm_next[d];
    const int32_t val = val_next;
    const float2 phv = ph_next;
    float4 rec[4];
    if constexpr (LP) {
#pragma unroll
      for (int q = 0; q < 4; ++q) rec[q] = rec_next[q];
    }
    if (r + 1 < nrounds) {
      i_next = it.start + min(s + PPB, it.len - 1);
      val_next = a.vals[i_next];
      if constexpr (LP) {
#pragma unroll
        for (int q = 0; q < 4; ++q) rec_next[q] = reinterpret_cast<const float4*>(pfr + i_next * 16)[q];
      } else {
        ph_next = ph[i_next];
      }
#pragma unroll
      for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
    }
    int base[D], local[D];
    const bool ok = point_base_at<float, D>(geo, tmv, jc.origin, base, local);
    float2 hy[NJ], hx[NJ];
    if constexpr (!LP) {
      // the point's D*NJ table factors, split over its LPP lanes, exchanged in scratch
#pragma unroll
      for (int f = k; f < D * NJ; f += LPP) {
        const int d = f / NJ, j = f % NJ;
        const int kb = table_bin<float>(d == 0 ? tmv[0] : tmv[1], (d == 0 ? base[0] : base[1]) + j,
                                        sel<float, D>(geo.Lr, d), sel<int, D>(geo.center, d),
                                        sel<int, D>(geo.tmax, d));
        pscr[f] = table_entry<float>(sel<const float2*, D>(geo.tab, d), kb, sel<int, D>(geo.center, d),
                                     sel<bool, D>(geo.half, d));
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        hy[j] = pscr[j];
        hx[j] = pscr[NJ + j];
      }
      __syncwarp();
    }
    if (active && 2 * k < jc.ncl) {
      const int64_t m = val - jc.t * a.M;
      float2 y0, y1;
      if (ok) {
        float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
        const float4* prow = reinterpret_cast<const float4*>(patch + (local[0] * PX + local[1]) * CS) + k;
        if constexpr (LP) {
          const float mx[NJ] = {rec[0].x, rec[0].y, rec[0].z, rec[0].w, rec[1].x, rec[1].y};
          const float my[NJ] = {rec[1].z, rec[1].w, rec[2].x, rec[2].y, rec[2].z, rec[2].w};
#pragma unroll
          for (int jy = 0; jy < NJ; ++jy) {
            float2 r0 = make_float2(0.f, 0.f), r1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx) {
              const float4 q = prow[(jy * PX + jx) * (CS / 2)];
              r0.x = fmaf(mx[jx], q.x, r0.x);
              r0.y = fmaf(mx[jx], q.y, r0.y);
              r1.x = fmaf(mx[jx], q.z, r1.x);
              r1.y = fmaf(mx[jx], q.w, r1.y);
            }
            acc0.x = fmaf(my[jy], r0.x, acc0.x);
            acc0.y = fmaf(my[jy], r0.y, acc0.y);
            acc1.x = fmaf(my[jy], r1.x, acc1.x);
            acc1.y = fmaf(my[jy], r1.y, acc1.y);
          }
          // conj(P Ey[ly - 1] Ex[lx - 1])
          const float2 Pc = cconj<float>(cmul<float>(
              make_float2(rec[3].x, rec[3].y),
              cmul<float>(etab[kLpE0 + local[0] - 1], etab[kLpEy + kLpE0 + local[1] - 1])));
          y0 = cmul<float>(acc0, Pc);
          y1 = cmul<float>(acc1, Pc);
        } else {
#pragma unroll
          for (int jy = 0; jy < NJ; ++jy) {
            float2 r0 = make_float2(0.f, 0.f), r1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int jx = 0; jx < NJ; ++jx) {
              const float4 q = prow[(jy * PX + jx) * (CS / 2)];
              r0 = cfma<float>(hx[jx], make_float2(q.x, q.y), r0);
              r1 = cfma<float>(hx[jx], make_float2(q.z, q.w), r1);
            }
            acc0 = cfma<float>(hy[jy], r0, acc0);
            acc1 = cfma<float>(hy[jy], r1, acc1);
          }
          y0 = cmul<float>(acc0, phv);
          y1 = cmul<float>(acc1, phv);
        }
      } else {
        y0 = y1 = make_float2(NAN, NAN);
      }
      float2* out = kdata + (jc.b * a.C + jc.c0 + 2 * k) * a.M + m;
      out[0] = y0;
      if (2 * k + 1 < jc.ncl) out[a.M] = y1;
    }
    if (active && !ok && k == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
  }
}

// LP: pfr = the pre-pass records, followed (at float2 offset 12 n) by the
// {Ey, Ex} tables, which each CTA copies behind its patch and factor scratch.
template <int CC, bool LP>
__global__ void __launch_bounds__(kThreads) k_interp_fwd_pairs(Geo<float> geo, Launch a, const float* __restrict__ tm,
                                                               const float2* __restrict__ ph,
                                                               const float2* __restrict__ grid,
                                                               float2* __restrict__ kdata,
                                                               const float* __restrict__ pfr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* patch = reinterpret_cast<float2*>(smem_raw);
  float2* etab = nullptr;
  if constexpr (LP) {
    constexpr int PPW = 64 / CC;
    etab = patch + a.cells * pair_cell_stride<CC>() + kWarps * PPW * 2 * 6;
    if (threadIdx.x < kLpEy + kLpEx) etab[threadIdx.x] = reinterpret_cast<const float2*>(pfr)[a.n * 12 + threadIdx.x];
    __syncthreads();
  }
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    fwd_job_pairs<CC, LP>(geo, a, tm, ph, grid, kdata, job, nitems, patch, pfr, etab);
}

// Exact values of the points the linear-phase gather left out (P = 0 in their
// records): one thread per (listed point, batch item, coil) gathers its 36
// taps from the grid with the table factors, after the main pass.
// (the body: blocks blk of nblk take (point, batch, coil) triples by a grid stride)
__device__ __forceinline__ void fwd_lp_fix_body(const Geo<float>& geo, const Launch& a, const float* __restrict__ tm,
                                                const float2* __restrict__ ph, const float2* __restrict__ grid,
                                                const int32_t* __restrict__ fix, const int32_t* __restrict__ nfix,
                                                float2* __restrict__ kdata, int64_t blk, int64_t nblk) {
  constexpr int D = 2, NJ = 6;
  const int64_t nb = a.ntraj == 1 ? a.B : 1;
  const int64_t total = (int64_t)(*nfix) * nb * a.C;
  for (int64_t w = blk * blockDim.x + threadIdx.x; w < total; w += nblk * blockDim.x) {
    const int64_t c = w % a.C, r = w / a.C;
    const int64_t i = fix[r / nb];
    const int32_t val = a.vals[i];
    const int64_t t = val / a.M, m = val - t * a.M;
    const int64_t b = a.ntraj == 1 ? r % nb : t;
    float2 hy[NJ], hx[NJ];
    int gy[NJ], gx[NJ];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float tv = tm[d * a.n + i];
      const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
      const float Lr = sel<float, D>(geo.Lr, d);
      const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d);
      const float2* tab = sel<const float2*, D>(geo.tab, d);
      const bool half = sel<bool, D>(geo.half, d);
      const int K = sel<int, D>(geo.K, d);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const float2 te = table_entry<float>(tab, table_bin<float>(tv, base + j, Lr, center, tmax), center, half);
        if (d == 0) {
          hy[j] = te;
          gy[j] = wrap_cell(base + j, K);
        } else {
          hx[j] = te;
          gx[j] = wrap_cell(base + j, K);
        }
      }
    }
    const float2* plane = grid + (b * a.C + c) * a.gtot;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      const float2* row = plane + (int64_t)gy[jy] * geo.K[1];
      float2 rs = make_float2(0.f, 0.f);
#pragma unroll
      for (int jx = 0; jx < NJ; ++jx) rs = cfma<float>(hx[jx], row[gx[jx]], rs);
      acc = cfma<float>(hy[jy], rs, acc);
    }
    kdata[(b * a.C + c) * a.M + m] = cmul<float>(acc, ph[i]);
  }
}

__global__ void __launch_bounds__(kThreads) k_fwd_lp_fix(Geo<float> geo, Launch a, const float* __restrict__ tm,
                                                         const float2* __restrict__ ph,
                                                         const float2* __restrict__ grid,
                                                         const int32_t* __restrict__ fix,
                                                         const int32_t* __restrict__ nfix, float2* __restrict__ kdata) {
  fwd_lp_fix_body(geo, a, tm, ph, grid, fix, nfix, kdata, blockIdx.x, gridDim.x);
}

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_interp_fwd(Geo<R> geo, Launch a, const R* __restrict__ tm,
                                                         const cplx<R>* __restrict__ ph,
                                                         const cplx<R>* __restrict__ grid, cplx<R>* __restrict__ kdata) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    fwd_job<R, D, JC>(geo, a, tm, ph, grid, kdata, job, nitems, patch);
}

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_interp_adj(Geo<R> geo, Launch a, const R* __restrict__ tm,
                                                         const cplx<R>* __restrict__ ph,
                                                         const cplx<R>* __restrict__ kdata, cplx<R>* __restrict__ grid) {
  constexpr int NJ = NJOf<JC>::N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* pre = reinterpret_cast<R*>(smem_raw);
  R* pim = pre + a.Cc * a.ps;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  cplx<R>* scr_warp = reinterpret_cast<cplx<R>*>(pre + 2 * a.Cc * a.ps) + warp * a.scratch;
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * kWarps;
  const int c = lane % a.Cc;
  const int pslot = lane / a.Cc;
  const bool coop = a.Cc >= 4;
  cplx<R>* scr = scr_warp + pslot * (D * NJ);
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    Item it;
    JobCtx jc;
    next_job<R>(geo, a, job, nitems, &it, &jc);
    __syncthreads();
    for (int idx = threadIdx.x; idx < 2 * a.Cc * a.ps; idx += kThreads) pre[idx] = R(0);
    __syncthreads();
    const int nrounds = (it.len + ppb - 1) / ppb;
    for (int r = 0; r < nrounds; ++r) {
      const int s = r * ppb + warp * ppw + pslot;
      const bool active = s < it.len;
      const int64_t i = it.start + (active ? s : 0);
      R tmv[D];
      int base[D], local[D];
      const bool ok = point_base<R, D>(geo, tm, a.n, i, jc.origin, tmv, base, local);
      cplx<R> h[D][NJ];
      table_factors<R, D, JC>(geo, tmv, base, c, a.Cc, coop, scr, h);
      if (active && ok && c < jc.ncl) {
        const int64_t m = a.vals[i] - jc.t * a.M;
        const cplx<R> v = cmulc<R>(kdata[(jc.b * a.C + jc.c0 + c) * a.M + m], ph[i]);
        scatter_point<R, D, JC>(geo, h, local, v, pre + c * a.ps, pim + c * a.ps);
      }
      if (active && !ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
    __syncthreads();
    flush_patch<R, D>(geo, grid, jc.b * a.C + jc.c0, a.gtot, jc.ncl, a.cells, a.ps, a.Cc, jc.origin, pre, pim);
  }
}

// ---------------------------------------------------------------------------
// K4 (owned tiles): atomic-free, deterministic adjoint.
//
// A CTA owns one output tile (T cells per dim, no halo) of Cc coil planes and
// accumulates, in shared memory, every point whose footprint reaches the tile:
// the points of the tile itself and of the nsrc-1 tiles before it in each
// dim. Points are taken in batches of kNB: the CTA first compacts the batch to
// the points that reach the tile and stages their conjugated table factors
// and phase-corrected k-space values; then each warp applies the batch to the
// rows of the tile it owns (disjoint rows: plain read-modify-write, no
// atomics; each cell sees its points in a fixed order). The tile is written
// once with coalesced stores, so the grid needs no zeroing.
// Requires K_d >= T_d + J_d - 1 (a footprint meets a tile in one run).

constexpr int kNB = 96;  // staged points per batch (multiple of 32, <= kThreads)

struct OwnLaunch {
  const Item* jobs;         // sub-jobs {tile key, first candidate, candidates, split}, longest first
  const int64_t* hdr;       // hdr[1] = number of sub-jobs
  const int32_t* counts;    // points per key
  const int32_t* tile_off;  // first sorted point of each key
  const int32_t* vals;
  int64_t n, M, ntraj, B, C;
  int Cc, ncc;
  int64_t nbpt;
  int aps;  // accumulator plane stride (complex elements)
  int64_t gtot;
  SrcSpan span;
  const int4* vlist;     // 2D: per-tile lists of the points that reach the tile (else null)
  const int32_t* voff;   // first list entry of each tile key
  const int32_t* koff;   // 2D lists sorted by footprint start: first entry of each start (else null)
  const float2* pfac;    // 2D register adjoint: per sorted point, 12 conjugated table factors (else null)
  const int4* vsort;     // 2D: each list chunk sorted by footprint start (else null)
};

template <typename R, int D>
__device__ __forceinline__ void own_tile_geometry(const Geo<R>& geo, int key, int64_t* t, int* td, int* origin,
                                                  int* ext) {
  *t = key / geo.ntiles;
  int rem = (int)(key - *t * geo.ntiles);
#pragma unroll
  for (int d = kMaxDim - 1; d >= 0; --d) {
    td[d] = 0;
    origin[d] = 0;
    ext[d] = 1;
    if (d < D) {
      td[d] = rem % geo.ntile[d];
      rem /= geo.ntile[d];
      origin[d] = td[d] * geo.T[d];
      ext[d] = min(geo.T[d], geo.K[d] - origin[d]);
    }
  }
}

// Zero the output tiles that are split over several sub-jobs (they are
// accumulated with atomics); every plane of the batch items the tile serves.
// Zero output tile it.key in every plane of the batch items it serves; the
// warps of CTA (x, y) take rows y*8 + warp, strided by 8*gridDim.y.
template <typename R, int D>
__device__ __forceinline__ void zero_tile(const Geo<R>& geo, const OwnLaunch& a, const Item& it,
                                          cplx<R>* __restrict__ grid) {
  int64_t t;
  int td[kMaxDim], origin[kMaxDim], ext[kMaxDim];
  own_tile_geometry<R, D>(geo, it.key, &t, td, origin, ext);
  const int64_t b0 = a.ntraj == 1 ? 0 : t, b1 = a.ntraj == 1 ? a.B : t + 1;
  int rows = 1;
#pragma unroll
  for (int d = 0; d < D - 1; ++d) rows *= ext[d];
  const int64_t nrow = (b1 - b0) * a.C * rows;
  const int64_t wstride = (int64_t)gridDim.y * (blockDim.x / 32);
  for (int64_t r = (int64_t)blockIdx.y * (blockDim.x / 32) + threadIdx.x / 32; r < nrow; r += wstride) {
    const int64_t plane = b0 * a.C + r / rows;
    int rr = (int)(r % rows);
    int64_t off = 0;
    if (D == 2) off = (int64_t)(origin[0] + rr) * geo.K[1];
    if (D == 3) {
      const int y = rr % ext[1 % D], z = rr / ext[1 % D];
      off = ((int64_t)(origin[0] + z) * geo.K[1 % D] + origin[1 % D] + y) * geo.K[2 % D];
    }
    cplx<R>* dst = grid + plane * a.gtot + off + origin[D - 1];
    for (int x = threadIdx.x & 31; x < ext[D - 1]; x += 32) dst[x] = mk<R>(0, 0);
  }
}

template <typename R, int D>
__global__ void k_zero_split_tiles(Geo<R> geo, OwnLaunch a, int W, cplx<R>* __restrict__ grid) {
  const int64_t nsj = a.hdr[1];
  for (int64_t j = blockIdx.x; j < nsj; j += gridDim.x) {
    const Item it = a.jobs[j];
    // sub-jobs are sorted longest first and a split tile's first sub-job
    // has the full length W: nothing after the first shorter job is one
    if (it.len < W) break;
    if (!(it.pad && it.start == 0)) continue;
    zero_tile<R, D>(geo, a, it, grid);
  }
}

// FAST: D == 2, J == 6, Cc == 16 and 16-row tiles — each warp owns two rows,
// lanes are (coil, row) and the six footprint columns are unrolled.
// One owned-tile adjoint job (a sub-job of one batch item and coil chunk).
// All threads of the CTA call it; smem_raw is the dynamic shared memory.
template <typename R, int D, int JC, bool FAST>
__device__ __forceinline__ void own_job(const Geo<R>& geo, const OwnLaunch& a, const R* __restrict__ tm,
                                        const cplx<R>* __restrict__ ph, const cplx<R>* __restrict__ kdata,
                                        cplx<R>* __restrict__ grid, int64_t job, unsigned char* smem_raw) {
  constexpr int NJ = NJOf<JC>::N;
  constexpr int MAXCOMBO = D == 1 ? 8 : (D == 2 ? 16 : 27);
  cplx<R>* acc = reinterpret_cast<cplx<R>*>(smem_raw);  // [Cc][aps]
  cplx<R>* sfac = acc + a.Cc * a.aps;                    // [kNB][D*NJ], conjugated
  cplx<R>* sv = sfac + kNB * D * NJ;                     // [kNB][Cc]
  int* sloc = reinterpret_cast<int*>(sv + kNB * a.Cc);   // [kNB][D] footprint start relative to the tile
  int* spt = sloc + kNB * D;                             // [kNB] sorted point index
  int* slist = spt + kNB;                                // [MAXCOMBO] list starts
  int* spre = slist + MAXCOMBO;                          // [MAXCOMBO + 1] candidate prefix
  int* snv = spre + MAXCOMBO + 1;                        // [kNB/32] valid count per staging warp

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t per_sj = a.nbpt * a.ncc;
  const int G = 32 / a.Cc;                       // lane groups per coil
  const int c = lane % a.Cc, grp = lane / a.Cc;  // this lane's coil and group
  const int JX = JC > 0 ? JC : geo.J[D - 1];
  const int cpg = (JX + G - 1) / G;              // footprint columns per group (generic path)
  int trows = 1;
#pragma unroll
  for (int d = 0; d < D - 1; ++d) trows *= geo.T[d];
  const int r_lo = FAST ? 2 * warp : (warp * trows) / kWarps;
  const int r_hi = FAST ? 2 * warp + 2 : ((warp + 1) * trows) / kWarps;
  const int TX = geo.T[D - 1];

  {
    const Item it = a.jobs[job / per_sj];
    const int64_t rest = job % per_sj;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    int64_t t;
    int td[kMaxDim], origin[kMaxDim], ext[kMaxDim];
    own_tile_geometry<R, D>(geo, it.key, &t, td, origin, ext);
    const int64_t b = a.ntraj == 1 ? bb : t;
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)a.Cc, a.C - c0);
    __syncthreads();  // previous job's write-out done with acc / lists
    if (threadIdx.x < a.span.ncombo) {
      const int skey = (int)(t * geo.ntiles) + source_tile(geo, a.span, td, threadIdx.x);
      slist[threadIdx.x] = a.tile_off[skey];
      spre[threadIdx.x + 1] = a.counts[skey];
    }
    if (threadIdx.x == 0) spre[0] = 0;
    for (int idx = threadIdx.x; idx < a.Cc * a.aps; idx += kThreads) acc[idx] = mk<R>(0, 0);
    __syncthreads();
    if (threadIdx.x == 0)
      for (int l = 0; l < a.span.ncombo; ++l) spre[l + 1] += spre[l];
    __syncthreads();
    const int qend = it.start + it.len;

    const int64_t vbase = a.vlist ? (int64_t)a.voff[it.key] : 0;
    for (int q0 = it.start; q0 < qend; q0 += kNB) {
      int nv = 0;
      if (D > 1 && a.vlist) {
        // A1 (2D, 3D): the tile's list holds only points that reach it
        nv = min(kNB, qend - q0);
        for (int e = threadIdx.x; e < nv; e += kThreads) {
          const int4 ent = a.vlist[vbase + q0 + e];
          spt[e] = ent.x;
          sloc[e * D] = ent.z;
          if (D == 2) {
            sloc[e * D + (D - 1)] = ent.w;
          } else {
            sloc[e * D + 1 % D] = (int)(short)(ent.w & 0xffff);
            sloc[e * D + 2 % D] = ent.w >> 16;
          }
        }
        __syncthreads();
      } else {
        // A1: which candidates reach the tile; compact them (two staging warps)
        if (warp < kNB / 32) {
          const int q = q0 + threadIdx.x;
          bool valid = false;
          int i = 0, rel[kMaxDim] = {0, 0, 0};
          if (q < qend) {
            int l = 0;
            while (spre[l + 1] <= q) ++l;
            i = slist[l] + (q - spre[l]);
            valid = true;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const R tv = tm[d * a.n + i];
              const R f = floor(sub_rn(tv, geo.halfJ[d]));
              const bool fin = fabs(f) < R(1 << 30);
              const int w = fin ? wrap_cell(1 + (int)f, geo.K[d]) : 0;
              int r = w - origin[d];
              if (r >= geo.T[d]) r -= geo.K[d];
              const int J = JC > 0 ? JC : geo.J[d];
              valid = valid && fin && (r > -J) && (r < ext[d]);
              rel[d] = r;
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, valid);
          if (lane == 0) snv[warp] = __popc(bal);
          __syncwarp();
          // named barrier 1 over the kNB staging threads only
          asm volatile("bar.sync 1, %0;" ::"r"(kNB));
          int pos = __popc(bal & ((1u << lane) - 1));
          for (int w = 0; w < warp; ++w) pos += snv[w];
          if (valid) {
            spt[pos] = i;
#pragma unroll
            for (int d = 0; d < D; ++d) sloc[pos * D + d] = rel[d];
          }
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < kNB / 32; ++w) nv += snv[w];
      }
      // A2: conjugated table factors (one thread per point and dim) and
      // conj(phase) * kdata of the staged points
      for (int e = threadIdx.x; e < nv * D; e += kThreads) {
        const int p = e / D;
        const int d = e - p * D;
        const int J = JC > 0 ? JC : sel<int, 3>(geo.J, d);
        const R tv = tm[d * a.n + spt[p]];
        const int base = 1 + (int)floor(sub_rn(tv, sel<R, 3>(geo.halfJ, d)));
        const R Lr = sel<R, 3>(geo.Lr, d);
        const int center = sel<int, 3>(geo.center, d), tmax = sel<int, 3>(geo.tmax, d);
        const cplx<R>* tab = sel<const cplx<R>*, 3>(geo.tab, d);
        const bool half = sel<bool, 3>(geo.half, d);
        cplx<R>* out = sfac + e * NJ;
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
          cplx<R> v = mk<R>(0, 0);
          if (JC > 0 || j < J) v = cconj<R>(table_entry<R>(tab, table_bin<R>(tv, base + j, Lr, center, tmax), center, half));
          out[j] = v;
        }
      }
      for (int e = threadIdx.x; e < nv * a.Cc; e += kThreads) {
        const int p = e / a.Cc;
        const int cl = e - p * a.Cc;
        cplx<R> v = mk<R>(0, 0);
        if (cl < ncl) {
          const int i = spt[p];
          const int64_t m = a.vals[i] - t * a.M;
          v = cmulc<R>(kdata[(b * a.C + c0 + cl) * a.M + m], ph[i]);
        }
        sv[e] = v;
      }
      __syncthreads();
      // B: each warp applies the staged points that touch its rows; a ballot
      // over the staged points (one lane per point) builds the warp's list.
      unsigned touch[kNB / 32];
#pragma unroll
      for (int h = 0; h < kNB / 32; ++h) {
        const int p = h * 32 + lane;
        bool tch = false;
        if (p < nv) {
          const int* loc = sloc + p * D;
          if (D == 1) {
            tch = warp == 0;
          } else if (D == 2) {
            const int JY = JC > 0 ? JC : geo.J[0];
            tch = max(0, r_lo - loc[0]) < min(JY, min(r_hi, ext[0]) - loc[0]);
          } else {
            const int JZ = JC > 0 ? JC : geo.J[0];
            const int JY = JC > 0 ? JC : geo.J[1 % D];
            const int T1 = geo.T[1 % D];
            const int y0 = max(loc[1 % D], 0), y1 = min(loc[1 % D] + JY, ext[1 % D]);
            for (int jz = 0; jz < JZ && !tch; ++jz) {
              const int z = loc[0] + jz;
              if (z < 0 || z >= ext[0] || y0 >= y1) continue;
              tch = max(z * T1 + y0, r_lo) < min(z * T1 + y1, r_hi);
            }
          }
        }
        touch[h] = __ballot_sync(0xffffffffu, tch);
      }
      if (FAST) {
        const int myrow = r_lo + grp;
        const bool rowok = myrow < ext[0];
#pragma unroll
        for (int h = 0; h < kNB / 32; ++h)
          for (unsigned msk = touch[h]; msk; msk &= msk - 1) {
            const int p = h * 32 + __ffs(msk) - 1;
            const int ly = sloc[p * 2], lx = sloc[p * 2 + 1];
            const int jy = myrow - ly;
            if (rowok && (unsigned)jy < 6u) {
              const cplx<R>* fp = sfac + p * 12;
              const cplx<R> vy = cmul<R>(sv[p * 16 + c], fp[jy]);
              cplx<R>* row = acc + c * a.aps + myrow * TX + lx;
              if (lx >= 0 && lx + 6 <= ext[1]) {  // footprint row fully inside the tile
#pragma unroll
                for (int jx = 0; jx < 6; ++jx) row[jx] = cfma<R>(vy, fp[6 + jx], row[jx]);
              } else {
#pragma unroll
                for (int jx = 0; jx < 6; ++jx)
                  if ((unsigned)(lx + jx) < (unsigned)ext[1]) row[jx] = cfma<R>(vy, fp[6 + jx], row[jx]);
              }
            }
          }
      } else {
#pragma unroll
        for (int h = 0; h < kNB / 32; ++h)
          for (unsigned msk = touch[h]; msk; msk &= msk - 1) {
            const int p = h * 32 + __ffs(msk) - 1;
            const int* loc = sloc + p * D;
            const cplx<R>* fp = sfac + p * D * NJ;
            const cplx<R> v = sv[p * a.Cc + c];
            if (D == 1) {
              for (int k = 0; k < cpg; ++k) {
                const int jx = grp * cpg + k;
                const int x = loc[0] + jx;
                if (jx < JX && x >= 0 && x < ext[0]) {
                  cplx<R>* cell = acc + c * a.aps + x;
                  *cell = cfma<R>(v, fp[jx], *cell);
                }
              }
            } else if (D == 2) {
              const int JY = JC > 0 ? JC : geo.J[0];
              const int jlo = max(0, r_lo - loc[0]);
              const int jhi = min(JY, min(r_hi, ext[0]) - loc[0]);
              for (int jy = jlo; jy < jhi; ++jy) {
                const cplx<R> vy = cmul<R>(v, fp[jy]);
                cplx<R>* row = acc + c * a.aps + (loc[0] + jy) * TX;
                for (int k = 0; k < cpg; ++k) {
                  const int jx = grp * cpg + k;
                  const int x = loc[1] + jx;
                  if (jx < JX && x >= 0 && x < ext[1]) row[x] = cfma<R>(vy, fp[NJ + jx], row[x]);
                }
              }
            } else {
              const int JZ = JC > 0 ? JC : geo.J[0];
              const int JY = JC > 0 ? JC : geo.J[1 % D];
              const int T1 = geo.T[1 % D];
              for (int jz = 0; jz < JZ; ++jz) {
                const int z = loc[0] + jz;
                if (z < 0 || z >= ext[0]) continue;
                const cplx<R> vz = cmul<R>(v, fp[jz]);
                for (int jy = 0; jy < JY; ++jy) {
                  const int y = loc[1 % D] + jy;
                  const int rr = z * T1 + y;
                  if (y < 0 || y >= ext[1 % D] || rr < r_lo || rr >= r_hi) continue;
                  const cplx<R> vy = cmul<R>(vz, fp[NJ + jy]);
                  cplx<R>* row = acc + c * a.aps + rr * TX;
                  for (int k = 0; k < cpg; ++k) {
                    const int jx = grp * cpg + k;
                    const int x = loc[2 % D] + jx;
                    if (jx < JX && x >= 0 && x < ext[2 % D]) row[x] = cfma<R>(vy, fp[2 * NJ + jx], row[x]);
                  }
                }
              }
            }
          }
      }
      __syncthreads();
    }
    // C: write the tile (rows of TX cells, coalesced); split tiles add atomically
    const bool split = it.pad != 0;
    for (int r = warp; r < ncl * trows; r += kWarps) {
      const int cl = r / trows;
      const int rr = r - cl * trows;
      int64_t off = 0;
      bool inside = true;
      if (D == 2) {
        inside = rr < ext[0];
        off = (int64_t)(origin[0] + rr) * geo.K[1];
      } else if (D == 3) {
        const int z = rr / geo.T[1 % D], y = rr - (rr / geo.T[1 % D]) * geo.T[1 % D];
        inside = z < ext[0] && y < ext[1 % D];
        off = ((int64_t)(origin[0] + z) * geo.K[1 % D] + origin[1 % D] + y) * geo.K[2 % D];
      }
      if (!inside) continue;
      cplx<R>* dst = grid + (b * a.C + c0 + cl) * a.gtot + off + origin[D - 1];
      const cplx<R>* src = acc + cl * a.aps + rr * TX;
      if (split) {
        for (int x = lane; x < ext[D - 1]; x += 32) atomic_add_global(&dst[x], src[x]);
      } else {
        for (int x = lane; x < ext[D - 1]; x += 32) dst[x] = src[x];
      }
    }
  }
}

template <typename R, int D, int JC, bool FAST>
__global__ void __launch_bounds__(kThreads) k_interp_adj_own(Geo<R> geo, OwnLaunch a, const R* __restrict__ tm,
                                                             const cplx<R>* __restrict__ ph,
                                                             const cplx<R>* __restrict__ kdata,
                                                             cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t njobs = a.hdr[1] * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    own_job<R, D, JC, FAST>(geo, a, tm, ph, kdata, grid, job, smem_raw);
}

// Smooth table lookup for the gradient: linear interpolation of value and
// derivative tables at the exact (unrounded) position.
// K4 (owned tiles, registers): the common 2D case — J = 6 in both dims,
// 16 coils per job, 16 x 14 tiles, complex64. Lane (coil c, row 2*warp + g)
// keeps the 14 cells of its row of its coil plane in registers. The tile's
// point list is sorted by footprint start (column offset, then row offset),
// so the points of one column offset that reach a warp's rows are one run of
// the list: a loop per column offset, unrolled over the 19 offsets, updates
// registers with static indices and needs no per-point branch; accumulation
// needs no shared-memory read-modify-write. Points are staged 256 at a time,
// two barriers per batch. Cells outside the tile (edge tiles narrower than 14) accumulate
// contributions that are never written; those cells belong to the wrapped
// tile, which gets the same points with its own column offsets.
constexpr int kNBR = 256;  // staged points per batch (== kThreads)
static_assert(kNBR == kListChunk, "a 2D register-adjoint batch is one sorted list chunk");
constexpr int kSVS = kNBR + 1;  // coil stride of the staged k-space values (bank spread)

// racc[LX + jx] += vy * fx[jx] for the columns inside the row (TXR cells).
template <int TXR, int LX>
__device__ __forceinline__ void reg_add_cols(float2 (&racc)[TXR], float2 vy, const float2 (&fx)[6]) {
#pragma unroll
  for (int jx = 0; jx < 6; ++jx)
    if (LX + jx >= 0 && LX + jx < TXR) racc[LX + jx] = cfma<float>(vy, fx[jx], racc[LX + jx]);
}

// The six conjugated table factors of sorted point i in dim d (2D, J = 6);
// the row factors (d = 0) carry conj(phase) as well.
__device__ __forceinline__ void reg_point_factors(const Geo<float>& geo, const float* __restrict__ tm,
                                                  const float2* __restrict__ ph, int64_t n, int64_t i, int d,
                                                  float2* out) {
  constexpr int D = 2, NJ = 6;
  const float tv = tm[d * n + i];
  const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
  const float Lr = sel<float, D>(geo.Lr, d);
  const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d);
  const float2* tab = sel<const float2*, D>(geo.tab, d);
  const bool half = sel<bool, D>(geo.half, d);
  const float2 phv = d == 0 ? ph[i] : make_float2(1.f, 0.f);
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float2 te = table_entry<float>(tab, table_bin<float>(tv, base + j, Lr, center, tmax), center, half);
    out[j] = cconj<float>(d == 0 ? cmul<float>(te, phv) : te);
  }
}

// Least-squares slopes of the D dims' table phases over u = k / L in (0, 1]
// (the whole block of kThreads threads; every thread gets c[0 .. D)).
template <int D>
__device__ __forceinline__ void lp_slopes_block(const Geo<float>& geo, double (&c)[D]) {
  __shared__ double s_red[2 * D][kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[2 * D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    acc[2 * d] = acc[2 * d + 1] = 0.0;
    const int center = sel<int, D>(geo.center, d), L = sel<int, D>(geo.L, d);
    const float2* tab = sel<const float2*, D>(geo.tab, d);
    const bool half = sel<bool, D>(geo.half, d);
    for (int k = 1 + (int)threadIdx.x; k <= L; k += kThreads) {
      const float2 h = table_entry<float>(tab, center + k, center, half);
      const double u = (double)k / (double)L;
      acc[2 * d] += u * (double)atan2f(h.y, h.x);
      acc[2 * d + 1] += u * u;
    }
  }
#pragma unroll
  for (int q = 0; q < 2 * D; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    if (lane == 0) s_red[q][warp] = acc[q];
  }
  __syncthreads();
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double su = 0.0, suu = 0.0;
    for (int w = 0; w < kWarps; ++w) {
      su += s_red[2 * d][w];
      suu += s_red[2 * d + 1][w];
    }
    c[d] = su / suu;
  }
  __syncthreads();
}

// Per sorted point i, dim d (thread pair 2i, 2i + 1): {mx[6], my[6], P} with
// P = conj(phase hy^[2] hx^[2]) (16 floats); returns this dim's h^[2].
__device__ __forceinline__ float2 reg_point_factors_lp(const Geo<float>& geo, const float* __restrict__ tm,
                                                       int64_t n, int64_t i, int d, float* out, bool* off) {
  constexpr int D = 2, NJ = 6;
  const float tv = tm[d * n + i];
  const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
  const float Lr = sel<float, D>(geo.Lr, d);
  const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d);
  const float2* tab = sel<const float2*, D>(geo.tab, d);
  const bool half = sel<bool, D>(geo.half, d);
  float* m = out + (d == 0 ? NJ : 0);  // mx first: 16-byte aligned for the adjoint's loads
  float2 hat = make_float2(1.f, 0.f);
  const int L = sel<int, D>(geo.L, d);
  int k0 = 0;
  bool mis = false;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int k = table_bin<float>(tv, base + j, Lr, center, tmax);
    if (j == 0) k0 = k;
    // the bins step by exactly L unless fl(tm - g) rounded (|tm| within a few
    // cells of 0): then this tap's phase is not the linear form's
    mis = mis || (k != k0 - j * L);
    const float2 te = table_entry<float>(tab, k, center, half);
    m[j] = sqrtf(te.x * te.x + te.y * te.y);
    if (j == 2) hat = make_float2(te.x / m[j], te.y / m[j]);
  }
  *off = mis;
  return hat;
}

// Pre-pass of the 2D register adjoint: every sorted point's factors once
// (a point sits in 1.8 tile lists on average), so the adjoint's staging is
// plain 16-byte copies. LP: the linear-phase form (16 floats per point).
// etab (LP): {Ey[kLpEy], Ex[kLpEx]}, written by block 0 (warp d fits dim
// d's phase slope, its lanes evaluate E_d[n] = e^{-i c n} in double).
// Points whose bins do not step by exactly L (see reg_point_factors_lp) get
// P = 0 (no contribution in the register adjoint) and go to `fix` (count in
// *nfix, reset by the host), whose exact contributions k_adj_lp_fix adds.
template <bool LP>
__global__ void __launch_bounds__(kThreads) k_point_factors2(Geo<float> geo, const float* __restrict__ tm,
                                                             const float2* __restrict__ ph, int64_t n,
                                                             float2* __restrict__ pfac, float2* __restrict__ etab,
                                                             int32_t* __restrict__ fix, int32_t* __restrict__ nfix) {
  if constexpr (LP) {
    if (blockIdx.x == 0) {
      double c[2];
      lp_slopes_block<2>(geo, c);
      const int t = threadIdx.x;
      if (t < kLpEy + kLpEx) {
        const bool y = t < kLpEy;
        double sn, cs;
        sincos((y ? c[0] : c[1]) * (double)((y ? t : t - kLpEy) - kLpE0), &sn, &cs);
        etab[t] = make_float2((float)cs, (float)-sn);
      }
    }
    // one thread per point, both dims (no exchange between lanes)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      float* rec = reinterpret_cast<float*>(pfac) + i * 16;
      bool mis_y = false, mis_x = false;
      const float2 hy = reg_point_factors_lp(geo, tm, n, i, 0, rec, &mis_y);
      const float2 hx = reg_point_factors_lp(geo, tm, n, i, 1, rec, &mis_x);
      float2 P = cmul<float>(cmul<float>(ph[i], hy), hx);
      if (mis_y || mis_x) {
        P = make_float2(0.f, 0.f);
        fix[atomicAdd(nfix, 1)] = (int32_t)i;
      }
      rec[12] = P.x;
      rec[13] = -P.y;
      rec[14] = 0.f;
      rec[15] = 0.f;
    }
  } else {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 2 * n;
         e += (int64_t)gridDim.x * blockDim.x)
      reg_point_factors(geo, tm, ph, n, e >> 1, (int)(e & 1), pfac + e * 6);
  }
}

// Exact contributions of the points the linear-phase adjoint left out: one
// thread per (listed point, batch item, coil) adds its 36 taps with vector
// atomics, after the register adjoint has written its tiles.
// (the body: blocks blk of nblk take (point, batch, coil) triples by a grid stride)
__device__ __forceinline__ void adj_lp_fix_body(const Geo<float>& geo, const OwnLaunch& a,
                                                const float* __restrict__ tm, const float2* __restrict__ ph,
                                                const float2* __restrict__ kdata, const int32_t* __restrict__ fix,
                                                const int32_t* __restrict__ nfix, float2* __restrict__ grid,
                                                int64_t blk, int64_t nblk) {
  constexpr int D = 2, NJ = 6;
  const int64_t nb = a.ntraj == 1 ? a.B : 1;
  const int64_t total = (int64_t)(*nfix) * nb * a.C;
  for (int64_t w = blk * blockDim.x + threadIdx.x; w < total; w += nblk * blockDim.x) {
    const int64_t c = w % a.C, r = w / a.C;
    const int64_t i = fix[r / nb];
    const int32_t val = a.vals[i];
    const int64_t t = val / a.M, m = val - t * a.M;
    const int64_t b = a.ntraj == 1 ? r % nb : t;
    float2 hy[NJ], hx[NJ];
    int gy[NJ], gx[NJ];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float tv = tm[d * a.n + i];
      const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
      const float Lr = sel<float, D>(geo.Lr, d);
      const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d);
      const float2* tab = sel<const float2*, D>(geo.tab, d);
      const bool half = sel<bool, D>(geo.half, d);
      const int K = sel<int, D>(geo.K, d);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const float2 te =
            cconj<float>(table_entry<float>(tab, table_bin<float>(tv, base + j, Lr, center, tmax), center, half));
        if (d == 0) {
          hy[j] = te;
          gy[j] = wrap_cell(base + j, K);
        } else {
          hx[j] = te;
          gx[j] = wrap_cell(base + j, K);
        }
      }
    }
    const float2 v = cmulc<float>(kdata[(b * a.C + c) * a.M + m], ph[i]);
    float2* plane = grid + (b * a.C + c) * a.gtot;
#pragma unroll
    for (int jy = 0; jy < NJ; ++jy) {
      const float2 vy = cmul<float>(v, hy[jy]);
#pragma unroll
      for (int jx = 0; jx < NJ; ++jx)
        atomic_add_global(plane + (int64_t)gy[jy] * geo.K[1] + gx[jx], cmul<float>(vy, hx[jx]));
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_adj_lp_fix(Geo<float> geo, OwnLaunch a, const float* __restrict__ tm,
                                                         const float2* __restrict__ ph,
                                                         const float2* __restrict__ kdata,
                                                         const int32_t* __restrict__ fix,
                                                         const int32_t* __restrict__ nfix, float2* __restrict__ grid) {
  adj_lp_fix_body(geo, a, tm, ph, kdata, fix, nfix, grid, blockIdx.x, gridDim.x);
}

// Footprint starts of a 16 x 14 tile with J = 6: row offsets -5 .. 15 (21),
// column offsets -5 .. 13 (19); start k = (rx + 5) * 21 + ry + 5.
constexpr int kRegKeyRows = kRegTileY + 5, kRegKeys = kRegKeyRows * (kRegTileX + 5);

// Points of the batch with column offset LXI - 5 that reach rows
// [r_lo, r_hi): positions ko[k(LXI, r_lo - 5)] .. ko[k(LXI, r_hi - 1) + 1] of
// the batch's sorted chunk; sloc[p] = (row offset, list position of its
// k-space values). With point groups (NG > 1) group g takes p = g mod NG.
template <int CC, int NG, int LXI>
__device__ __forceinline__ void reg_columns(const int32_t* ko, int r_lo, int r_hi,
                                           int grp, const float2* __restrict__ sfac, const float2* __restrict__ sv,
                                           const int2* __restrict__ sloc, int myrow, bool rowok, int c,
                                           float2 (&racc)[kRegTileX]) {
  constexpr int NJ = 6, LX = LXI - 5;
  const int kb = LXI * kRegKeyRows;
  int p = ko[kb + r_lo];
  const int e = ko[kb + r_hi + 5];
  if (NG > 1) p += (grp - p % NG + NG) % NG;
  // two entries per iteration: their shared-memory loads are in flight together
#pragma unroll 2
  for (; p < e; p += NG) {
    const int2 lp = sloc[p];
    const int jy = myrow - lp.x;
    const float2* fp = sfac + p * (2 * NJ);
    float2 fy = make_float2(0.f, 0.f);
    if (rowok && (unsigned)jy < (unsigned)NJ) fy = fp[jy];
    const float2 vy = cmul<float>(sv[c * kSVS + lp.y], fy);
    const float4* fx4 = reinterpret_cast<const float4*>(fp + NJ);
    const float4 f01 = fx4[0], f23 = fx4[1], f45 = fx4[2];
    const float2 fx[6] = {make_float2(f01.x, f01.y), make_float2(f01.z, f01.w), make_float2(f23.x, f23.y),
                          make_float2(f23.z, f23.w), make_float2(f45.x, f45.y), make_float2(f45.z, f45.w)};
    reg_add_cols<kRegTileX, LX>(racc, vy, fx);
  }
  if constexpr (LXI + 1 < kRegTileX + 5)
    reg_columns<CC, NG, LXI + 1>(ko, r_lo, r_hi, grp, sfac, sv, sloc, myrow, rowok, c, racc);
}

// racc[LX + jx] += vy * m[jx] for the columns inside the row (real factors).
template <int TXR, int LX>
__device__ __forceinline__ void reg_add_cols_real(float2 (&racc)[TXR], float2 vy, const float (&m)[6]) {
#pragma unroll
  for (int jx = 0; jx < 6; ++jx)
    if (LX + jx >= 0 && LX + jx < TXR) {
      racc[LX + jx].x = fmaf(vy.x, m[jx], racc[LX + jx].x);
      racc[LX + jx].y = fmaf(vy.y, m[jx], racc[LX + jx].y);
    }
}

// End of the 2D register adjoint's staging buffers (shared memory): the
// linear-phase E tables follow.
__host__ __device__ constexpr size_t reg_rtab_offset(int CC) {
  return (size_t)kNBR * 2 * 6 * sizeof(float2) + (size_t)CC * kSVS * sizeof(float2) + (size_t)kNBR * sizeof(int2) +
         (size_t)(kRegKeys + 1) * sizeof(int32_t);
}

// Linear-phase form of reg_columns: sfr[p] = {mx[6], my[6]} (48 bytes), the
// staged k-space values already carry Q.
template <int CC, int NG, int LXI>
__device__ __forceinline__ void reg_columns_lp(const int32_t* ko, int r_lo, int r_hi, int grp,
                                              const float* __restrict__ sfr, const float2* __restrict__ sv,
                                              const int2* __restrict__ sloc, int myrow, bool rowok, int c,
                                              float2 (&racc)[kRegTileX]) {
  constexpr int NJ = 6, LX = LXI - 5;
  const int kb = LXI * kRegKeyRows;
  int p = ko[kb + r_lo];
  const int e = ko[kb + r_hi + 5];
  if (NG > 1) p += (grp - p % NG + NG) % NG;
  // two entries per iteration: their shared-memory loads are in flight together
#pragma unroll 2
  for (; p < e; p += NG) {
    const int2 lp = sloc[p];
    const int jy = myrow - lp.x;
    const float* fp = sfr + p * (2 * NJ);
    float my = 0.f;
    if (rowok && (unsigned)jy < (unsigned)NJ) my = fp[NJ + jy];
    const float2 v = sv[c * kSVS + lp.y];
    const float2 vy = make_float2(v.x * my, v.y * my);
    const float4 m03 = *reinterpret_cast<const float4*>(fp);
    const float2 m45 = *reinterpret_cast<const float2*>(fp + 4);
    const float m[6] = {m03.x, m03.y, m03.z, m03.w, m45.x, m45.y};
    reg_add_cols_real<kRegTileX, LX>(racc, vy, m);
  }
  if constexpr (LXI + 1 < kRegTileX + 5)
    reg_columns_lp<CC, NG, LXI + 1>(ko, r_lo, r_hi, grp, sfr, sv, sloc, myrow, rowok, c, racc);
}

// vec_ok: the grid pointer is 16-byte aligned and K1 is even, so every
// tile row starts 16-byte aligned and pairs of cells go out as one float4.
// CC coils per job (2, 4, 8 or 16; one coil runs as CC = 2 with the second
// masked). A warp covers RPW = 32 / CC tile rows with lanes (coil, row); WPT =
// 16 / RPW warps cover the tile, and the kWarps / WPT groups of warps take
// the staged points in turn (point p goes to group p mod NG). With more than
// one group, the groups' partial tiles are summed in a fixed order through
// shared memory before the write-out, so results stay deterministic.
// tmap (or null): the grid as a 3D tensor (2 K1 floats, K0 rows, B C planes)
// with a box of one tile of CC planes; whole unsplit tiles of CC coils are
// then written by one tensor store from shared memory.
// LP: linear-phase tables (see kLpE0): real factors from the pre-pass,
// k-space values times Q per list entry, tile times R; etab = {Ey[kLpEy],
// Ex[kLpEx]} in shared memory (set up by the kernel).
template <int CC, bool LP = false>
__device__ __forceinline__ void reg_job(const Geo<float>& geo, const OwnLaunch& a, const float* __restrict__ tm,
                                        const float2* __restrict__ ph, const float2* __restrict__ kdata,
                                        float2* __restrict__ grid, int vec_ok, int64_t job, unsigned char* smem_raw,
                                        const CUtensorMap* tmap, const float2* etab = nullptr) {
  constexpr int D = 2, NJ = 6;
  constexpr int RPW = 32 / CC, WPT = kRegTileY / RPW, NG = kWarps / WPT;
  static_assert(CC >= 2 && CC <= 16 && (CC & (CC - 1)) == 0, "coils per job");
  float2* sfac = reinterpret_cast<float2*>(smem_raw);  // [kNBR][12]: conj y factors (times conj phase), conj x
  float2* sv = sfac + kNBR * D * NJ;                   // [CC][kSVS] kdata, in list order
  int2* sloc = reinterpret_cast<int2*>(sv + CC * kSVS);  // [kNBR] (row offset, list position), sorted order
  float2* part = reinterpret_cast<float2*>(smem_raw);    // [NG][16][14][CC] partial tiles (after the batches)

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = lane % CC, grp = warp / WPT;
  const int myrow = (warp % WPT) * RPW + lane / CC;
  const int64_t per_sj = a.nbpt * a.ncc;

  {
    const Item it = a.jobs[job / per_sj];
    const int64_t rest = job % per_sj;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    int64_t t;
    int td[kMaxDim], origin[kMaxDim], ext[kMaxDim];
    own_tile_geometry<float, D>(geo, it.key, &t, td, origin, ext);
    const int64_t b = a.ntraj == 1 ? bb : t;
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)min(CC, a.Cc), a.C - c0);
    const bool rowok = myrow < ext[0];
    const int64_t vbase = a.voff[it.key];
    int32_t* ko = reinterpret_cast<int32_t*>(sloc + kNBR);  // [kRegKeys + 1] the batch's run starts
    float2 racc[kRegTileX];
#pragma unroll
    for (int x = 0; x < kRegTileX; ++x) racc[x] = make_float2(0.f, 0.f);
    const int qend = it.start + it.len;
    // The staging buffers are free here: the previous batch ended with a barrier.
    for (int q0 = it.start; q0 < qend; q0 += kNBR) {
      const int nv = min(kNBR, qend - q0);
      // A: the batch is one chunk of the tile's list. Thread s copies entry s's
      // k-space values of every coil (list order: a warp's 32 entries are
      // mostly runs of consecutive m, so its copies touch few lines); the
      // chunk's sorted copy gives, per sorted position, the footprint start,
      // the list position and the table factors; ko = its run starts.
      const int4* ents = a.vlist + vbase + q0;
      const int4* sents = a.vsort + vbase + q0;
      {
        const int64_t krow = (vbase + q0) / kListChunk + it.key;
        for (int k = threadIdx.x; k <= kRegKeys; k += kThreads) ko[k] = a.koff[krow * (kRegKeys + 1) + k];
      }
      if ((int)threadIdx.x < nv) {
        const int s = threadIdx.x;
        const float2* src = kdata + (b * a.C + c0) * a.M + ents[s].y;
#pragma unroll 4
        for (int cl = 0; cl < CC; ++cl) {
          if (cl < ncl)
            cp_async_elem(sv + cl * kSVS + s, src + cl * a.M);
          else
            sv[cl * kSVS + s] = make_float2(0.f, 0.f);
        }
      }
      if (LP) {
        // the point's real factors {mx[6], my[6]}: three 16-byte copies of its record
        for (int e = threadIdx.x; e < nv * 3; e += kThreads) {
          const int pt = e / 3, q = e - pt * 3;
          const int4 ent = sents[pt];
          if (q == 0) sloc[pt] = make_int2(ent.z, ent.y);
          cp_async_16(sfac + pt * NJ + 2 * q, a.pfac + (int64_t)ent.x * 8 + 2 * q);
        }
      } else if (a.pfac) {
        // the point's 12 factors, precomputed per sorted point: six 16-byte copies
        for (int e = threadIdx.x; e < nv * 6; e += kThreads) {
          const int pt = e / 6, q = e - pt * 6;
          const int4 ent = sents[pt];
          if (q == 0) sloc[pt] = make_int2(ent.z, ent.y);
          cp_async_16(sfac + pt * (D * NJ) + 2 * q, a.pfac + (int64_t)ent.x * (D * NJ) + 2 * q);
        }
      } else {
        for (int e = threadIdx.x; e < nv * D; e += kThreads) {
          const int pt = e >> 1, d = e & 1;
          const int4 ent = sents[pt];
          if (d == 0) sloc[pt] = make_int2(ent.z, ent.y);
          reg_point_factors(geo, tm, ph, a.n, ent.x, d, sfac + e * NJ);
        }
      }
      cp_async_wait_all();
      if (LP && (int)threadIdx.x < nv) {
        // this thread's own copies have landed: the entry's values times
        // Q = P Ey[2 + ry] Ex[2 + rx]
        const int s = threadIdx.x;
        const int4 ent = ents[s];
        const float2 P = a.pfac[(int64_t)ent.x * 8 + 6];
        const float2 Q =
            cmul<float>(P, cmul<float>(etab[kLpE0 + 2 + ent.z], etab[kLpEy + kLpE0 + 2 + ent.w]));
#pragma unroll 4
        for (int cl = 0; cl < CC; ++cl) sv[cl * kSVS + s] = cmul<float>(sv[cl * kSVS + s], Q);
      }
      __syncthreads();
      // B: the list is sorted by footprint start (column offset, then row
      // offset), so for each column offset LX the points that reach this
      // warp's rows [r_lo, r_hi) — row offsets r_lo - 5 .. r_hi - 1 — are one
      // run of the batch; LX is a template argument, so every update uses
      // static register indices. Lanes whose row the footprint misses add 0.
      {
        const int r_lo = (warp % WPT) * RPW, r_hi = min(r_lo + RPW, ext[0]);
        if (r_lo < r_hi) {
          if constexpr (LP)
            reg_columns_lp<CC, NG, 0>(ko, r_lo, r_hi, grp, reinterpret_cast<const float*>(sfac), sv, sloc, myrow,
                                      rowok, c, racc);
          else
            reg_columns<CC, NG, 0>(ko, r_lo, r_hi, grp, sfac, sv, sloc, myrow, rowok, c, racc);
        }
      }
      __syncthreads();
    }
    const int ex = ext[1];
    if constexpr (LP) {
      // the tile-cell phase R(y, x) = conj(Ey[y] Ex[x]) (tile-local y, x)
      const float2 ey = cconj<float>(etab[kLpE0 + myrow]);
#pragma unroll
      for (int x = 0; x < kRegTileX; ++x)
        racc[x] = cmul<float>(racc[x], cmul<float>(ey, cconj<float>(etab[kLpEy + kLpE0 + x])));
    }
    if (NG == 1) {
      // C: whole unsplit tiles of CC coils go out as one tensor store (the
      // staging buffers are free after the last batch's barrier; rows and
      // columns past the grid edge fall outside the tensor and are dropped);
      // otherwise each lane writes its row, split tiles adding atomically
      if (tmap && it.pad == 0 && ncl == CC && ((uintptr_t)smem_raw & 127) == 0) {
        float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float2*>(smem_raw) +
                                                (c * kRegTileY + myrow) * kRegTileX);
#pragma unroll
        for (int x = 0; x < kRegTileX; x += 2)
          dst[x / 2] = make_float4(racc[x].x, racc[x].y, racc[x + 1].x, racc[x + 1].y);
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
          tma_store_3d(tmap, smem_raw, 2 * origin[1], origin[0], (int)(b * a.C + c0));
          bulk_commit();
          bulk_wait_read();
        }
        __syncthreads();
      } else if (rowok && c < ncl) {
        float2* dst = grid + (b * a.C + c0 + c) * a.gtot + (int64_t)(origin[0] + myrow) * geo.K[1] + origin[1];
        if (it.pad == 0) {
          if (vec_ok) {
#pragma unroll
            for (int x = 0; x < kRegTileX; x += 2) {
              if (x + 1 < ex)
                *reinterpret_cast<float4*>(dst + x) = make_float4(racc[x].x, racc[x].y, racc[x + 1].x, racc[x + 1].y);
              else if (x < ex)
                dst[x] = racc[x];
            }
          } else {
#pragma unroll
            for (int x = 0; x < kRegTileX; ++x)
              if (x < ex) dst[x] = racc[x];
          }
        } else {
#pragma unroll
          for (int x = 0; x < kRegTileX; ++x)
            if (x < ex) atomic_add_global(dst + x, racc[x]);
        }
      }
    } else {
      // C: the groups' partial tiles meet in shared memory (the staging
      // buffers are free after the last batch's barrier); thread e sums
      // element e (coil-major, then row, then column) over the groups in order
      constexpr int TE = kRegTileY * kRegTileX * CC;
#pragma unroll
      for (int x = 0; x < kRegTileX; ++x) part[grp * TE + (c * kRegTileY + myrow) * kRegTileX + x] = racc[x];
      __syncthreads();
      for (int e = threadIdx.x; e < TE; e += kThreads) {
        const int cl = e / (kRegTileY * kRegTileX);
        const int rr = (e / kRegTileX) % kRegTileY, x = e % kRegTileX;
        if (cl >= ncl || rr >= ext[0] || x >= ex) continue;
        float2 v = part[e];
#pragma unroll
        for (int q = 1; q < NG; ++q) {
          const float2 w = part[q * TE + e];
          v.x += w.x;
          v.y += w.y;
        }
        float2* dst = grid + (b * a.C + c0 + cl) * a.gtot + (int64_t)(origin[0] + rr) * geo.K[1] + origin[1] + x;
        if (it.pad == 0)
          *dst = v;
        else
          atomic_add_global(dst, v);
      }
      __syncthreads();  // the next job's staging reuses the buffer
    }
  }
}

// K4 (owned tiles, registers), 3D: complex64, J = 6, 4 x 8 x 8 tiles, CC
// coils per job (2, 4 or 8; one coil runs as CC = 2). Lane (coil, z, y) keeps
// the 8 x-cells of one (z, y) row of the tile in registers; a warp covers all
// 4 z planes of 32 / (4 CC) y rows, so with the tile's list sorted by
// (x offset, y offset) the points reaching a warp's rows are one run per x
// offset, as in the 2D kernel. The groups of warps that cover the tile take
// the staged points in turn.
constexpr int kReg3Z = 4, kReg3Y = 8, kReg3X = 8, kReg3Rows = kReg3Z * kReg3Y;
// footprint starts (y, x) of a 4 x 8 x 8 tile with J = 6: 13 x 13
constexpr int kReg3KeyRows = kReg3Y + 5, kReg3Keys = kReg3KeyRows * (kReg3X + 5);

// Points of the batch with x offset LXI - 5 whose y rows reach [ylo, yhi):
// positions ko[k(LXI, ylo - 5)] .. ko[k(LXI, yhi - 1) + 1] of the batch's
// sorted chunk; sloc[p] = (z offset, y offset, list position of its values).
template <int CC, int NG, int LXI>
__device__ __forceinline__ void reg3_columns(const int32_t* ko, int ylo, int yhi, int grp,
                                            const float2* __restrict__ sfac, const float2* __restrict__ sv,
                                            const int4* __restrict__ sloc, int mz, int my, bool rowok, int c,
                                            float2 (&racc)[kReg3X]) {
  constexpr int NJ = 6, LX = LXI - 5;
  const int kb = LXI * kReg3KeyRows;
  int p = ko[kb + ylo];
  const int e = ko[kb + yhi + 5];
  if (NG > 1) p += (grp - p % NG + NG) % NG;
  // two entries per iteration: their shared-memory loads are in flight together
#pragma unroll 2
  for (; p < e; p += NG) {
    const int4 loc = sloc[p];
    const int jz = mz - loc.x, jy = my - loc.y;
    const float2* fp = sfac + p * (3 * NJ);
    float2 fz = make_float2(0.f, 0.f), fy = make_float2(0.f, 0.f);
    if (rowok && (unsigned)jz < (unsigned)NJ && (unsigned)jy < (unsigned)NJ) {
      fz = fp[jz];
      fy = fp[NJ + jy];
    }
    const float2 vzy = cmul<float>(cmul<float>(sv[c * kSVS + loc.z], fz), fy);
    const float4* fx4 = reinterpret_cast<const float4*>(fp + 2 * NJ);
    const float4 f01 = fx4[0], f23 = fx4[1], f45 = fx4[2];
    const float2 fx[6] = {make_float2(f01.x, f01.y), make_float2(f01.z, f01.w), make_float2(f23.x, f23.y),
                          make_float2(f23.z, f23.w), make_float2(f45.x, f45.y), make_float2(f45.z, f45.w)};
    reg_add_cols<kReg3X, LX>(racc, vzy, fx);
  }
  if constexpr (LXI + 1 < kReg3X + 5)
    reg3_columns<CC, NG, LXI + 1>(ko, ylo, yhi, grp, sfac, sv, sloc, mz, my, rowok, c, racc);
}

// Linear-phase 3D: per sorted position 20 floats {mx[6], pad[2], my[6], mz[6]}
// (mx 16-byte aligned); E tables E_d[n], n = -kLp3E0 .. 9, per dim.
constexpr int kLp3Rec = 20, kLp3E0 = 3, kLp3En = 13;

template <int CC, int NG, int LXI>
__device__ __forceinline__ void reg3_columns_lp(const int32_t* ko, int ylo, int yhi, int grp,
                                               const float* __restrict__ sfr, const float2* __restrict__ sv,
                                               const int4* __restrict__ sloc, int mz, int my, bool rowok, int c,
                                               float2 (&racc)[kReg3X]) {
  constexpr int NJ = 6, LX = LXI - 5;
  const int kb = LXI * kReg3KeyRows;
  int p = ko[kb + ylo];
  const int e = ko[kb + yhi + 5];
  if (NG > 1) p += (grp - p % NG + NG) % NG;
  // two entries per iteration: their shared-memory loads are in flight together
#pragma unroll 2
  for (; p < e; p += NG) {
    const int4 loc = sloc[p];
    const int jz = mz - loc.x, jy = my - loc.y;
    const float* fp = sfr + p * kLp3Rec;
    float w = 0.f;
    if (rowok && (unsigned)jz < (unsigned)NJ && (unsigned)jy < (unsigned)NJ) w = fp[14 + jz] * fp[8 + jy];
    const float2 v = sv[c * kSVS + loc.z];
    const float2 vzy = make_float2(v.x * w, v.y * w);
    const float4 m03 = *reinterpret_cast<const float4*>(fp);
    const float2 m45 = *reinterpret_cast<const float2*>(fp + 4);
    const float m[6] = {m03.x, m03.y, m03.z, m03.w, m45.x, m45.y};
    reg_add_cols_real<kReg3X, LX>(racc, vzy, m);
  }
  if constexpr (LXI + 1 < kReg3X + 5)
    reg3_columns_lp<CC, NG, LXI + 1>(ko, ylo, yhi, grp, sfr, sv, sloc, mz, my, rowok, c, racc);
}

// Pre-pass of the 3D linear-phase register adjoint: per sorted point its 18
// real magnitudes where the adjoint stages them (x at 0, y at 8, z at 14)
// and at 20 the phase word conj(phase hz^[2] hy^[2] hx^[2]) (kLp3PRec floats
// per point), so the adjoint's staging is plain 16-byte copies. A point whose
// bins do not step by exactly L gets a zero phase word and is listed in lfix
// (count at 0, indices from 16; the count reset by the host) for
// k_adj_lp_fix3. One thread per point.
__global__ void __launch_bounds__(kThreads) k_point_factors3(Geo<float> geo, const float* __restrict__ tm,
                                                             const float2* __restrict__ ph, int64_t n,
                                                             float* __restrict__ rec3, int32_t* __restrict__ lfix) {
  constexpr int D = 3, NJ = 6;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float* rec = rec3 + i * kLp3PRec;
    float2 P = ph[i];
    bool mis = false;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float tv = tm[d * n + i];
      const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
      const float Lr = sel<float, D>(geo.Lr, d);
      const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d), L = sel<int, D>(geo.L, d);
      const float2* tab = sel<const float2*, D>(geo.tab, d);
      const bool half = sel<bool, D>(geo.half, d);
      const int k0 = table_bin<float>(tv, base, Lr, center, tmax);
      float* out = rec + (d == 2 ? 0 : (d == 1 ? 8 : 14));
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        const int kb = table_bin<float>(tv, base + j, Lr, center, tmax);
        // for |tm| >= 8, tm and every g are within a factor 2 of each other:
        // fl(tm - g) is exact and the bins step by exactly L
        mis = mis || (fabsf(tv) < 8.f && kb != k0 - j * L);
        const float2 te = table_entry<float>(tab, kb, center, half);
        out[j] = sqrtf(te.x * te.x + te.y * te.y);
      }
      const float2 te = table_entry<float>(tab, k0 - 2 * L, center, half);
      const float mg = sqrtf(te.x * te.x + te.y * te.y);
      P = cmul<float>(P, make_float2(te.x / mg, te.y / mg));
    }
    float2 Pc = cconj<float>(P);
    if (mis) {
      Pc = make_float2(0.f, 0.f);
      lfix[16 + atomicAdd(lfix, 1)] = (int32_t)i;
    }
    rec[6] = rec[7] = 0.f;
    rec[20] = Pc.x;
    rec[21] = Pc.y;
    rec[22] = rec[23] = 0.f;
  }
}

// End of the 3D register adjoint's staging buffers (the E tables follow).
__host__ __device__ constexpr size_t reg3_etab_offset(int CC) {
  return (((size_t)kNBR * 3 * 6 * sizeof(float2) + (size_t)CC * kSVS * sizeof(float2) + (size_t)kNBR * sizeof(int4) +
           (size_t)(kReg3Keys + 1) * sizeof(int32_t)) + 7) & ~(size_t)7;
}

// LP (linear-phase tables, see kLpE0): real kernel values per sorted
// position, k-space values times Q = conj(phase prod_d h_d^[2]) prod_d
// E_d[2 + r_d] per list entry, tile times R = conj(prod_d E_d[cell_d]);
// etab = {Ez, Ey, Ex} in shared memory. A point whose bins do not step by
// exactly L gets Q = 0 and, from the entry of the tile holding its first
// footprint cell, goes to lfix (count at 0, indices from 16) for the exact pass.
template <int CC, bool LP = false>
__device__ __forceinline__ void reg3_job(const Geo<float>& geo, const OwnLaunch& a, const float* __restrict__ tm,
                                         const float2* __restrict__ ph, const float2* __restrict__ kdata,
                                         float2* __restrict__ grid, int vec_ok, int64_t job, unsigned char* smem_raw,
                                         const float2* etab = nullptr, const float* __restrict__ rec3 = nullptr) {
  constexpr int D = 3, NJ = 6;
  // lane (coil, z, y): a warp covers all kReg3Z planes of YB rows y0 .. y0 + YB - 1
  constexpr int RPW = 32 / CC, YB = RPW / kReg3Z, WPT = kReg3Y / YB, NG = kWarps / WPT;
  static_assert(CC >= 2 && CC <= 8 && (CC & (CC - 1)) == 0, "coils per job");
  float2* sfac = reinterpret_cast<float2*>(smem_raw);  // [kNBR][18]: conj z (times conj phase), y, x factors
  float2* sv = sfac + kNBR * D * NJ;                   // [CC][kSVS] kdata, in list order
  int4* sloc = reinterpret_cast<int4*>(sv + CC * kSVS);  // [kNBR] (z offset, y offset, list position), sorted
  float2* part = reinterpret_cast<float2*>(smem_raw);    // [NG][CC][32][8] partial tiles (after the batches)

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = lane % CC, grp = warp / WPT;
  const int y0 = (warp % WPT) * YB;
  const int mz = (lane / CC) % kReg3Z, my = y0 + (lane / CC) / kReg3Z;
  const int myrow = mz * kReg3Y + my;
  const int64_t per_sj = a.nbpt * a.ncc;
  {
    const Item it = a.jobs[job / per_sj];
    const int64_t rest = job % per_sj;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    int64_t t;
    int td[kMaxDim], origin[kMaxDim], ext[kMaxDim];
    own_tile_geometry<float, D>(geo, it.key, &t, td, origin, ext);
    const int64_t b = a.ntraj == 1 ? bb : t;
    const int c0 = cc * a.Cc;
    const int ncl = (int)min((int64_t)min(CC, a.Cc), a.C - c0);
    const bool rowok = mz < ext[0] && my < ext[1];
    const int64_t vbase = a.voff[it.key];
    int32_t* ko = reinterpret_cast<int32_t*>(sloc + kNBR);  // [kReg3Keys + 1] the batch's run starts
    const int y_hi = min(y0 + YB, ext[1]);
    float2 racc[kReg3X];
#pragma unroll
    for (int x = 0; x < kReg3X; ++x) racc[x] = make_float2(0.f, 0.f);
    const int qend = it.start + it.len;
    for (int q0 = it.start; q0 < qend; q0 += kNBR) {
      const int nv = min(kNBR, qend - q0);
      // A: the batch is one chunk of the tile's list: k-space values copied in
      // list order (thread s: entry s, every coil), footprint starts, list
      // positions and conjugated table factors (z factors times conj(phase))
      // in the chunk's sorted order; ko = the chunk's run starts
      const int4* ents = a.vlist + vbase + q0;
      const int4* sents = a.vsort + vbase + q0;
      {
        const int64_t krow = (vbase + q0) / kListChunk + it.key;
        for (int k = threadIdx.x; k <= kReg3Keys; k += kThreads) ko[k] = a.koff[krow * (kReg3Keys + 1) + k];
      }
      if ((int)threadIdx.x < nv) {
        const int s = threadIdx.x;
        const float2* src = kdata + (b * a.C + c0) * a.M + ents[s].y;
#pragma unroll
        for (int cl = 0; cl < CC; ++cl) {
          if (cl < ncl)
            cp_async_elem(sv + cl * kSVS + s, src + cl * a.M);
          else
            sv[cl * kSVS + s] = make_float2(0.f, 0.f);
        }
      }
      if constexpr (LP) {
        // the sorted point's 18 magnitudes: five 16-byte copies of its pre-pass record
        for (int e = threadIdx.x; e < nv * 5; e += kThreads) {
          const int pt = e / 5, q = e - pt * 5;
          const int4 ent = sents[pt];
          if (q == 0) sloc[pt] = make_int4(ent.z, (int)(short)(ent.w & 0xffff), ent.y, 0);
          cp_async_16(sfac + pt * (kLp3Rec / 2) + 2 * q,
                      reinterpret_cast<const float2*>(rec3) + (int64_t)ent.x * (kLp3PRec / 2) + 2 * q);
        }
      }
      for (int e = threadIdx.x; e < (LP ? 0 : nv * D); e += kThreads) {
        const int pt = e / D, d = e - (e / D) * D;
        const int4 ent = sents[pt];
        if (d == 0) sloc[pt] = make_int4(ent.z, (int)(short)(ent.w & 0xffff), ent.y, 0);
        const float tv = tm[d * a.n + ent.x];
        const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
        const float Lr = sel<float, D>(geo.Lr, d);
        const int center = sel<int, D>(geo.center, d), tmax = sel<int, D>(geo.tmax, d);
        const float2* tab = sel<const float2*, D>(geo.tab, d);
        const bool half = sel<bool, D>(geo.half, d);
        if constexpr (LP) {
          // real magnitudes: x at 0, y at 8, z at 14 of the position's record
          float* out = reinterpret_cast<float*>(sfac) + pt * kLp3Rec + (d == 2 ? 0 : (d == 1 ? 8 : 14));
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            const float2 te = table_entry<float>(tab, table_bin<float>(tv, base + j, Lr, center, tmax), center, half);
            out[j] = sqrtf(te.x * te.x + te.y * te.y);
          }
        } else {
          const float2 phv = d == 0 ? ph[ent.x] : make_float2(1.f, 0.f);
          float2* out = sfac + e * NJ;
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            const float2 te = table_entry<float>(tab, table_bin<float>(tv, base + j, Lr, center, tmax), center, half);
            out[j] = cconj<float>(d == 0 ? cmul<float>(te, phv) : te);
          }
        }
      }
      cp_async_wait_all();
      if (LP && (int)threadIdx.x < nv) {
        // this thread's own copies have landed: entry s's values times
        // Q = (phase word of its point) * prod_d E_d[2 + r_d] (zero for a left-out point)
        const int s = threadIdx.x;
        const int4 ent = ents[s];
        const int r[3] = {ent.z, (int)(short)(ent.w & 0xffff), ent.w >> 16};
        float2 Q = reinterpret_cast<const float2*>(rec3)[(int64_t)ent.x * (kLp3PRec / 2) + 10];
#pragma unroll
        for (int d = 0; d < D; ++d) Q = cmul<float>(Q, etab[d * kLp3En + kLp3E0 + 2 + r[d]]);
#pragma unroll
        for (int cl = 0; cl < CC; ++cl) sv[cl * kSVS + s] = cmul<float>(sv[cl * kSVS + s], Q);
      }
      __syncthreads();
      // B: runs of the list sorted by (column offset, row offset): for each
      // column offset, the points whose rows reach y0 .. y_hi - 1
      if (y0 < y_hi) {
        if constexpr (LP)
          reg3_columns_lp<CC, NG, 0>(ko, y0, y_hi, grp, reinterpret_cast<const float*>(sfac), sv, sloc, mz, my,
                                     rowok, c, racc);
        else
          reg3_columns<CC, NG, 0>(ko, y0, y_hi, grp, sfac, sv, sloc, mz, my, rowok, c, racc);
      }
      __syncthreads();
    }
    const int ex = ext[2];
    if constexpr (LP) {
      // the tile-cell phase R(z, y, x) = conj(Ez[z] Ey[y] Ex[x]) (tile-local)
      const float2 ezy = cconj<float>(cmul<float>(etab[kLp3E0 + mz], etab[kLp3En + kLp3E0 + my]));
#pragma unroll
      for (int x = 0; x < kReg3X; ++x)
        racc[x] = cmul<float>(racc[x], cmul<float>(ezy, cconj<float>(etab[2 * kLp3En + kLp3E0 + x])));
    }
    if (NG == 1) {
      if (rowok && c < ncl) {
        float2* dst = grid + (b * a.C + c0 + c) * a.gtot +
                      ((int64_t)(origin[0] + mz) * geo.K[1] + origin[1] + my) * geo.K[2] + origin[2];
        if (it.pad == 0) {
          if (vec_ok) {
#pragma unroll
            for (int x = 0; x < kReg3X; x += 2) {
              if (x + 1 < ex)
                *reinterpret_cast<float4*>(dst + x) = make_float4(racc[x].x, racc[x].y, racc[x + 1].x, racc[x + 1].y);
              else if (x < ex)
                dst[x] = racc[x];
            }
          } else {
#pragma unroll
            for (int x = 0; x < kReg3X; ++x)
              if (x < ex) dst[x] = racc[x];
          }
        } else {
#pragma unroll
          for (int x = 0; x < kReg3X; ++x)
            if (x < ex) atomic_add_global(dst + x, racc[x]);
        }
      }
    } else {
      constexpr int TE = kReg3Rows * kReg3X * CC;
#pragma unroll
      for (int x = 0; x < kReg3X; ++x) part[grp * TE + (c * kReg3Rows + myrow) * kReg3X + x] = racc[x];
      __syncthreads();
      for (int e = threadIdx.x; e < TE; e += kThreads) {
        const int cl = e / (kReg3Rows * kReg3X);
        const int rr = (e / kReg3X) % kReg3Rows, x = e % kReg3X;
        const int z = rr / kReg3Y, y = rr % kReg3Y;
        if (cl >= ncl || z >= ext[0] || y >= ext[1] || x >= ex) continue;
        float2 v = part[e];
#pragma unroll
        for (int q = 1; q < NG; ++q) {
          const float2 w = part[q * TE + e];
          v.x += w.x;
          v.y += w.y;
        }
        float2* dst = grid + (b * a.C + c0 + cl) * a.gtot +
                      ((int64_t)(origin[0] + z) * geo.K[1] + origin[1] + y) * geo.K[2] + origin[2] + x;
        if (it.pad == 0)
          *dst = v;
        else
          atomic_add_global(dst, v);
      }
      __syncthreads();
    }
  }
}

template <int CC, bool LP>
__global__ void __launch_bounds__(kThreads, 3) k_interp_adj_reg3(Geo<float> geo, OwnLaunch a,
                                                                 const float* __restrict__ tm,
                                                                 const float2* __restrict__ ph,
                                                                 const float2* __restrict__ kdata,
                                                                 float2* __restrict__ grid, int vec_ok,
                                                                 const float* __restrict__ rec3) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* etab = reinterpret_cast<float2*>(smem_raw + reg3_etab_offset(CC));  // [3][kLp3En], past the staging
  if constexpr (LP) {
    // per CTA: the three dims' phase slopes (least squares) and E_d[n] = e^{-i c_d n} in double
    double c3[3];
    lp_slopes_block<3>(geo, c3);
    if (threadIdx.x < 3 * kLp3En) {
      const int d = threadIdx.x / kLp3En, nidx = threadIdx.x % kLp3En;
      double sn, cs;
      sincos(c3[d] * (double)(nidx - kLp3E0), &sn, &cs);
      etab[threadIdx.x] = make_float2((float)cs, (float)-sn);
    }
    __syncthreads();
  }
  const int64_t njobs = a.hdr[1] * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    reg3_job<CC, LP>(geo, a, tm, ph, kdata, grid, vec_ok, job, smem_raw, etab, rec3);
}

// Exact contributions of the points the 3D linear-phase adjoint left out
// (one thread per (listed point, batch item, coil), 216 taps with vector
// atomics), after the register pass.
__global__ void __launch_bounds__(kThreads) k_adj_lp_fix3(Geo<float> geo, OwnLaunch a, const float* __restrict__ tm,
                                                          const float2* __restrict__ ph,
                                                          const float2* __restrict__ kdata,
                                                          const int32_t* __restrict__ lfix,
                                                          float2* __restrict__ grid) {
  constexpr int D = 3, NJ = 6;
  const int64_t nb = a.ntraj == 1 ? a.B : 1;
  const int64_t total = (int64_t)lfix[0] * nb * a.C;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = w % a.C, r = w / a.C;
    const int64_t i = lfix[16 + r / nb];
    const int32_t val = a.vals[i];
    const int64_t t = val / a.M, m = val - t * a.M;
    const int64_t b = a.ntraj == 1 ? r % nb : t;
    float2 h[D][NJ];
    int g[D][NJ];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float tv = tm[d * a.n + i];
      const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        h[d][j] = cconj<float>(table_entry<float>(
            sel<const float2*, D>(geo.tab, d),
            table_bin<float>(tv, base + j, sel<float, D>(geo.Lr, d), sel<int, D>(geo.center, d),
                             sel<int, D>(geo.tmax, d)),
            sel<int, D>(geo.center, d), sel<bool, D>(geo.half, d)));
        g[d][j] = wrap_cell(base + j, sel<int, D>(geo.K, d));
      }
    }
    const float2 v = cmulc<float>(kdata[(b * a.C + c) * a.M + m], ph[i]);
    float2* plane = grid + (b * a.C + c) * a.gtot;
    for (int jz = 0; jz < NJ; ++jz) {
      const float2 vz = cmul<float>(v, h[0][jz]);
#pragma unroll
      for (int jy = 0; jy < NJ; ++jy) {
        const float2 vzy = cmul<float>(vz, h[1][jy]);
        const int64_t row = ((int64_t)g[0][jz] * geo.K[1] + g[1][jy]) * geo.K[2];
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx) atomic_add_global(plane + row + g[2][jx], cmul<float>(vzy, h[2][jx]));
      }
    }
  }
}

// ---------------------------------------------------------------- K3, 3D linear-phase
// Gather for 3D complex64, J = 6, 4 x 8 x 8 tiles (patch 9 x 13 x 13, fixed at
// compile time), linear-phase tables, with the layout of the generic gather:
// one shared-memory plane per coil, one lane per (point, coil). After staging,
// patch cell (Z, Y, X) is multiplied by Ez[Z - 3] Ey[Y - 3] Ex[X - 3]; a lane
// takes its point's 18 real magnitudes and phase word Pw from the point's
// pre-pass record (k_point_factors3) and does two real multiply-adds per tap:
//   y = conj(Pw prod_d E_d[l_d - 1]) sum prod_d m_d[j_d] X'(l + j),
// (l the footprint start in the patch; Pw = conj(phase prod_d h^_d[2])). A
// left-out point has Pw = 0 and is rewritten by k_fwd_lp_fix3. Every lane
// runs the taps; a point outside its tile reads the patch at its first cell
// and is written as NaN.
constexpr int kP3Z = kReg3Z + 5, kP3Y = kReg3Y + 5, kP3X = kReg3X + 5, kP3Cells = kP3Z * kP3Y * kP3X;
constexpr int kP3PS = kP3Cells | 1;  // plane stride (odd: a point's coil lanes hit distinct banks)

template <int CC>
__host__ __device__ constexpr size_t fwd_lp3_smem() {
  return (size_t)CC * kP3PS * sizeof(float2) + (size_t)3 * kLp3En * sizeof(float2);
}

template <int CC>
__device__ __forceinline__ void fwd_job_lp3(const Geo<float>& geo, const Launch& a, const float* __restrict__ tm,
                                            const float2* __restrict__ grid, float2* __restrict__ kdata, int64_t job,
                                            int64_t nitems, float2* patch, const float2* etab,
                                            const float* __restrict__ rec3) {
  constexpr int D = 3, NJ = 6, PPW = 32 / CC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = lane % CC, pslot = lane / CC;
  Item it;
  JobCtx jc;
  next_job<float>(geo, a, job, nitems, &it, &jc);
  __syncthreads();
  load_patch<float, D>(geo, grid, jc.b * a.C + jc.c0, a.gtot, jc.ncl, kP3Cells, kP3PS, jc.origin, patch);
  __syncthreads();
  // the patch times Ez[Z - 3] Ey[Y - 3] Ex[X - 3] (E_d[n] at etab[d kLp3En + kLp3E0 + n]):
  // thread per cell, every coil plane
  for (int cell = threadIdx.x; cell < kP3Cells; cell += kThreads) {
    const int Z = cell / (kP3Y * kP3X), rem = cell - Z * (kP3Y * kP3X);
    const int Y = rem / kP3X, X = rem - Y * kP3X;
    const float2 E = cmul<float>(cmul<float>(etab[Z], etab[kLp3En + Y]), etab[2 * kLp3En + X]);
#pragma unroll
    for (int cl = 0; cl < CC; ++cl) {
      float2* pc = patch + cl * kP3PS + cell;
      *pc = cmul<float>(*pc, E);
    }
  }
  __syncthreads();
  constexpr int PPB = PPW * kWarps;
  const int nrounds = (it.len + PPB - 1) / PPB;
  int64_t i_next = it.start + min(warp * PPW + pslot, it.len - 1);
  float tm_next[D];
  int32_t val_next = a.vals[i_next];
#pragma unroll
  for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
  for (int r = 0; r < nrounds; ++r) {
    const int s = r * PPB + warp * PPW + pslot;
    const bool active = s < it.len;
    const int64_t i = it.start + min(s, it.len - 1);
    float tmv[D];
#pragma unroll
    for (int d = 0; d < D; ++d) tmv[d] = tm_next[d];
    const int32_t val = val_next;
    if (r + 1 < nrounds) {
      i_next = it.start + min(s + PPB, it.len - 1);
      val_next = a.vals[i_next];
#pragma unroll
      for (int d = 0; d < D; ++d) tm_next[d] = tm[d * a.n + i_next];
    }
    int base[D], local[D];
    const bool ok = point_base_at<float, D>(geo, tmv, jc.origin, base, local);
    // the record: mx at 0, my at 8, mz at 14, Pw at 20
    const float4* rq = reinterpret_cast<const float4*>(rec3 + i * kLp3PRec);
    const float4 q0 = rq[0], q1 = rq[1], q2 = rq[2], q3 = rq[3], q4 = rq[4], q5 = rq[5];
    const float mx[NJ] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
    const float my[NJ] = {q2.x, q2.y, q2.z, q2.w, q3.x, q3.y};
    const float mz[NJ] = {q3.z, q3.w, q4.x, q4.y, q4.z, q4.w};
    const int lz = ok ? local[0] : 0, ly = ok ? local[1] : 0, lx = ok ? local[2] : 0;
    const float2* pp = patch + c * kP3PS + (lz * kP3Y + ly) * kP3X + lx;
    float ar = 0.f, ai = 0.f;
#pragma unroll
    for (int jz = 0; jz < NJ; ++jz) {
      float sr = 0.f, si = 0.f;
#pragma unroll
      for (int jy = 0; jy < NJ; ++jy) {
        float rr = 0.f, ri = 0.f;
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx) {
          const float2 v = pp[(jz * kP3Y + jy) * kP3X + jx];
          rr = fmaf(mx[jx], v.x, rr);
          ri = fmaf(mx[jx], v.y, ri);
        }
        sr = fmaf(my[jy], rr, sr);
        si = fmaf(my[jy], ri, si);
      }
      ar = fmaf(mz[jz], sr, ar);
      ai = fmaf(mz[jz], si, ai);
    }
    const float2 El = cmul<float>(cmul<float>(etab[kLp3E0 + lz - 1], etab[kLp3En + kLp3E0 + ly - 1]),
                                  etab[2 * kLp3En + kLp3E0 + lx - 1]);
    float2 y = cmulc<float>(make_float2(ar, ai), cmul<float>(make_float2(q5.x, q5.y), El));
    if (!ok) y = make_float2(NAN, NAN);
    if (active && c < jc.ncl) kdata[(jc.b * a.C + jc.c0 + c) * a.M + (val - jc.t * a.M)] = y;
    if (active && !ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
  }
}

template <int CC>
__global__ void __launch_bounds__(kThreads) k_interp_fwd_lp3(Geo<float> geo, Launch a, const float* __restrict__ tm,
                                                             const float2* __restrict__ grid,
                                                             float2* __restrict__ kdata, const float* __restrict__ rec3) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* patch = reinterpret_cast<float2*>(smem_raw);
  float2* etab = patch + CC * kP3PS;  // [3][kLp3En]
  {
    // per CTA: the three dims' phase slopes (least squares) and E_d[n] = e^{-i c_d n} in double
    double c3[3];
    lp_slopes_block<3>(geo, c3);
    if (threadIdx.x < 3 * kLp3En) {
      const int d = threadIdx.x / kLp3En, nidx = threadIdx.x % kLp3En;
      double sn, cs;
      sincos(c3[d] * (double)(nidx - kLp3E0), &sn, &cs);
      etab[threadIdx.x] = make_float2((float)cs, (float)-sn);
    }
    __syncthreads();
  }
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    fwd_job_lp3<CC>(geo, a, tm, grid, kdata, job, nitems, patch, etab, rec3);
}

// Exact values of the points the 3D linear-phase gather left out: one thread
// per (listed point, batch item, coil) gathers its 216 taps from the grid with
// the table factors.
__global__ void __launch_bounds__(kThreads) k_fwd_lp_fix3(Geo<float> geo, Launch a, const float* __restrict__ tm,
                                                          const float2* __restrict__ ph,
                                                          const float2* __restrict__ grid,
                                                          const int32_t* __restrict__ lfix, float2* __restrict__ kdata) {
  constexpr int D = 3, NJ = 6;
  const int64_t nb = a.ntraj == 1 ? a.B : 1;
  const int64_t total = (int64_t)lfix[0] * nb * a.C;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = w % a.C, r = w / a.C;
    const int64_t i = lfix[16 + r / nb];
    const int32_t val = a.vals[i];
    const int64_t t = val / a.M, m = val - t * a.M;
    const int64_t b = a.ntraj == 1 ? r % nb : t;
    float2 h[D][NJ];
    int g[D][NJ];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float tv = tm[d * a.n + i];
      const int base = 1 + (int)floorf(sub_rn(tv, sel<float, D>(geo.halfJ, d)));
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        h[d][j] = table_entry<float>(sel<const float2*, D>(geo.tab, d),
                                     table_bin<float>(tv, base + j, sel<float, D>(geo.Lr, d),
                                                      sel<int, D>(geo.center, d), sel<int, D>(geo.tmax, d)),
                                     sel<int, D>(geo.center, d), sel<bool, D>(geo.half, d));
        g[d][j] = wrap_cell(base + j, sel<int, D>(geo.K, d));
      }
    }
    const float2* plane = grid + (b * a.C + c) * a.gtot;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int jz = 0; jz < NJ; ++jz) {
      float2 az = make_float2(0.f, 0.f);
#pragma unroll
      for (int jy = 0; jy < NJ; ++jy) {
        const float2* row = plane + ((int64_t)g[0][jz] * geo.K[1] + g[1][jy]) * geo.K[2];
        float2 ay = make_float2(0.f, 0.f);
#pragma unroll
        for (int jx = 0; jx < NJ; ++jx) ay = cfma<float>(h[2][jx], row[g[2][jx]], ay);
        az = cfma<float>(h[1][jy], ay, az);
      }
      acc = cfma<float>(h[0][jz], az, acc);
    }
    kdata[(b * a.C + c) * a.M + m] = cmul<float>(acc, ph[i]);
  }
}

template <int CC, bool LP>
__global__ void __launch_bounds__(kThreads, 3)
    k_interp_adj_reg(Geo<float> geo, OwnLaunch a, const float* __restrict__ tm, const float2* __restrict__ ph,
                     const float2* __restrict__ kdata, float2* __restrict__ grid, int vec_ok, int use_tmap,
                     const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* etab = reinterpret_cast<float2*>(smem_raw + reg_rtab_offset(CC));  // {Ey, Ex}, past the staging
  if constexpr (LP) {
    // the phase tables written by the pre-pass, after the per-point records
    if (threadIdx.x < kLpEy + kLpEx) etab[threadIdx.x] = a.pfac[a.n * 12 + threadIdx.x];
    __syncthreads();
  }
  const int64_t njobs = a.hdr[1] * a.nbpt * a.ncc;
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x)
    reg_job<CC, LP>(geo, a, tm, ph, kdata, grid, vec_ok, job, smem_raw, use_tmap ? &tmap : nullptr, etab);
  if (use_tmap && threadIdx.x == 0) bulk_wait();  // every tensor store has completed
}

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
// y = phase * sum_j prod_d h_d(u_d) X[idx_j], u_d = tm_d - g_d, tm = omega/gam,
// d tm_d / d omega_d = 1 / gam_d and d phase / d omega_d = i n_shift_d phase.
// Uses the patch staging of the forward; one lane per (point, coil), coils
// reduced with warp shuffles, batches with atomics.
template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_interp_grad(Geo<R> geo, Launch a, const R* __restrict__ tm,
                                                          const cplx<R>* __restrict__ ph,
                                                          const cplx<R>* __restrict__ grid,
                                                          const cplx<R>* __restrict__ v, R* __restrict__ grad) {
  constexpr int NJ = NJOf<JC>::N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  const int64_t nitems = a.hdr[0];
  const int64_t njobs = nitems * a.nbpt * a.ncc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ppw = 32 / a.Cc;
  const int ppb = ppw * kWarps;
  const int c = lane % a.Cc;
  // with 4 or more coil lanes per point, the lanes split the 2*D*NJ value and
  // derivative factors of their point and exchange them through scratch
  const bool coop = a.Cc >= 4;
  cplx<R>* scr = patch + a.Cc * a.ps + (warp * ppw + lane / a.Cc) * (2 * D * NJ);
  for (int64_t job = blockIdx.x; job < njobs; job += gridDim.x) {
    Item it;
    JobCtx jc;
    next_job<R>(geo, a, job, nitems, &it, &jc);
    __syncthreads();
    load_patch<R, D>(geo, grid, jc.b * a.C + jc.c0, a.gtot, jc.ncl, a.cells, a.ps, jc.origin, patch);
    __syncthreads();
    const int nrounds = (it.len + ppb - 1) / ppb;
    for (int r = 0; r < nrounds; ++r) {
      const int s = r * ppb + warp * ppw + lane / a.Cc;
      const bool active = s < it.len;
      const int64_t i = it.start + (active ? s : 0);
      R tmv[D];
      int base[D], local[D];
      const bool ok = point_base<R, D>(geo, tm, a.n, i, jc.origin, tmv, base, local) && active;
      cplx<R> hv[D][NJ], hd[D][NJ];
      if (coop) {
        for (int f = c; f < D * NJ; f += a.Cc) {
          const int d = f / NJ, j = f - (f / NJ) * NJ;
          cplx<R> fv = mk<R>(0, 0), fd = mk<R>(0, 0);
          if (JC > 0 || j < sel<int, 3>(geo.J, d)) lerp_tables<R>(geo, d, sel<R, D>(tmv, d), sel<int, D>(base, d) + j, &fv, &fd);
          scr[f] = fv;
          scr[D * NJ + f] = fd;
        }
        __syncwarp();
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            hv[d][j] = scr[d * NJ + j];
            hd[d][j] = scr[D * NJ + d * NJ + j];
          }
        __syncwarp();
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) {
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            if (JC > 0 || j < geo.J[d]) {
              lerp_tables<R>(geo, d, tmv[d], base[d] + j, &hv[d][j], &hd[d][j]);
            } else {
              hv[d][j] = mk<R>(0, 0);
              hd[d][j] = mk<R>(0, 0);
            }
          }
        }
      }
      R gsum[D];
#pragma unroll
      for (int d = 0; d < D; ++d) gsum[d] = R(0);
      int64_t m = 0;
      if (ok) m = a.vals[i] - jc.t * a.M;
      if (ok && c < jc.ncl) {
        const cplx<R>* plane = patch + c * a.ps;
        cplx<R> val = mk<R>(0, 0);
        cplx<R> der[D];
#pragma unroll
        for (int d = 0; d < D; ++d) der[d] = mk<R>(0, 0);
        if (D == 1) {
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            if (JC > 0 || j < geo.J[0]) {
              const cplx<R> x = plane[local[0] + j];
              val = cfma<R>(hv[0][j], x, val);
              der[0] = cfma<R>(hd[0][j], x, der[0]);
            }
          }
        } else if (D == 2) {
#pragma unroll
          for (int jy = 0; jy < NJ; ++jy) {
            if (JC > 0 || jy < geo.J[0]) {
              cplx<R> rv = mk<R>(0, 0), rd = mk<R>(0, 0);
              const cplx<R>* row = plane + (local[0] + jy) * geo.P[1 % D] + local[1 % D];
#pragma unroll
              for (int jx = 0; jx < NJ; ++jx) {
                if (JC > 0 || jx < geo.J[1 % D]) {
                  const cplx<R> x = row[jx];
                  rv = cfma<R>(hv[1 % D][jx], x, rv);
                  rd = cfma<R>(hd[1 % D][jx], x, rd);
                }
              }
              val = cfma<R>(hv[0][jy], rv, val);
              der[0] = cfma<R>(hd[0][jy], rv, der[0]);
              der[1 % D] = cfma<R>(hv[0][jy], rd, der[1 % D]);
            }
          }
        } else {
#pragma unroll 1
          for (int jz = 0; jz < NJ; ++jz) {
            if (JC > 0 || jz < geo.J[0]) {
              cplx<R> zv = mk<R>(0, 0), zdy = mk<R>(0, 0), zdx = mk<R>(0, 0);
#pragma unroll
              for (int jy = 0; jy < NJ; ++jy) {
                if (JC > 0 || jy < geo.J[1 % D]) {
                  cplx<R> rv = mk<R>(0, 0), rd = mk<R>(0, 0);
                  const cplx<R>* row =
                      plane + ((local[0] + jz) * geo.P[1 % D] + local[1 % D] + jy) * geo.P[2 % D] + local[2 % D];
#pragma unroll
                  for (int jx = 0; jx < NJ; ++jx) {
                    if (JC > 0 || jx < geo.J[2 % D]) {
                      const cplx<R> x = row[jx];
                      rv = cfma<R>(hv[2 % D][jx], x, rv);
                      rd = cfma<R>(hd[2 % D][jx], x, rd);
                    }
                  }
                  zv = cfma<R>(hv[1 % D][jy], rv, zv);
                  zdy = cfma<R>(hd[1 % D][jy], rv, zdy);
                  zdx = cfma<R>(hv[1 % D][jy], rd, zdx);
                }
              }
              // jz is a runtime index, so hv[0][jz] is read through a select chain
              cplx<R> hz = hv[0][0], dz = hd[0][0];
#pragma unroll
              for (int q = 1; q < NJ; ++q)
                if (q == jz) {
                  hz = hv[0][q];
                  dz = hd[0][q];
                }
              val = cfma<R>(hz, zv, val);
              der[0] = cfma<R>(dz, zv, der[0]);
              der[1 % D] = cfma<R>(hz, zdy, der[1 % D]);
              der[2 % D] = cfma<R>(hz, zdx, der[2 % D]);
            }
          }
        }
        const cplx<R> p = ph[i];
        const cplx<R> vv = v[(jc.b * a.C + jc.c0 + c) * a.M + m];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          // dy/d omega_d = phase * (der_d / gam_d + i * nshift_d * val)
          const cplx<R> inner = mk<R>(der[d].x / geo.gam[d] - geo.nshift[d] * val.y,
                                      der[d].y / geo.gam[d] + geo.nshift[d] * val.x);
          const cplx<R> dy = cmul<R>(p, inner);
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
        for (int d = 0; d < D; ++d) atomicAdd(&grad[(jc.t * D + d) * a.M + m], gsum[d]);
      }
      if (active && !ok && c == 0) atomicOr(&g_status, kStatusNonFinite | kStatusOutsidePatch);
    }
  }
}

// ---------------------------------------------------------------- K8 ragged
// Many independent problems (each its own grid and image size, trajectory
// and coil count; one dtype, ndim and numpoints) in one launch per stage.
// Every entry of the merged, longest-first job list names its problem; a CTA
// copies that problem's descriptor into shared memory when the problem
// changes and runs the same per-job code as the single-problem kernels.
template <typename R>
struct RaggedProb {
  Geo<R> geo;
  Launch a;
  OwnLaunch o;
  const R* tm;
  const cplx<R>* ph;
  cplx<R>* grid;
  cplx<R>* kdata;
  int64_t nitems;
  int vec_ok;
  int lp;                 // linear-phase problem: the register adjoint and coil-pair gather in the real form
  const float2* etab;     // lp: {Ey, Ex} in the problem's workspace
  const int32_t* fix;     // lp: the left-out points and their count
  const int32_t* nfix;
};

template <typename T>
__device__ __forceinline__ void load_desc(T* dst, const T* __restrict__ src) {
  static_assert(sizeof(T) % 4 == 0, "descriptor size");
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x) d[i] = s[i];
}

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_ragged_fwd(const RaggedProb<R>* __restrict__ probs,
                                                         const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<R> sp;
  cplx<R>* patch = reinterpret_cast<cplx<R>*>(smem_raw);
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      __syncthreads();
      cur = pj.x;
    }
    fwd_job<R, D, JC>(sp.geo, sp.a, sp.tm, sp.ph, sp.grid, sp.kdata, pj.y, sp.nitems, patch);
  }
}

template <int CC>
__global__ void __launch_bounds__(kThreads) k_ragged_fwd_pairs(const RaggedProb<float>* __restrict__ probs,
                                                               const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<float> sp;
  float2* patch = reinterpret_cast<float2*>(smem_raw);
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      __syncthreads();
      cur = pj.x;
    }
    fwd_job_pairs<CC, false>(sp.geo, sp.a, sp.tm, sp.ph, sp.grid, sp.kdata, pj.y, sp.nitems, patch);
  }
}

template <typename R, int D>
__global__ void k_ragged_zero(const RaggedProb<R>* __restrict__ probs, const int2* __restrict__ jobs, int64_t njobs) {
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    const RaggedProb<R>& P = probs[pj.x];
    zero_tile<R, D>(P.geo, P.o, P.o.jobs[pj.y], P.grid);
  }
}

template <int CC>
__global__ void __launch_bounds__(kThreads, 3) k_ragged_adj_reg(const RaggedProb<float>* __restrict__ probs,
                                                                const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<float> sp;
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      __syncthreads();
      cur = pj.x;
    }
    reg_job<CC>(sp.geo, sp.o, sp.tm, sp.ph, sp.kdata, sp.grid, sp.vec_ok, pj.y, smem_raw, nullptr);
  }
}

// Linear-phase problems (RaggedProb::lp): the same per-job code in the real
// form; a CTA also copies the problem's E tables when the problem changes.
template <int CC>
__global__ void __launch_bounds__(kThreads, 3) k_ragged_fwd_pairs_lp(const RaggedProb<float>* __restrict__ probs,
                                                                  const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<float> sp;
  __shared__ float2 setab[kLpEy + kLpEx];
  float2* patch = reinterpret_cast<float2*>(smem_raw);
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      if (threadIdx.x < kLpEy + kLpEx) setab[threadIdx.x] = probs[pj.x].etab[threadIdx.x];
      __syncthreads();
      cur = pj.x;
    }
    fwd_job_pairs<CC, true>(sp.geo, sp.a, sp.tm, sp.ph, sp.grid, sp.kdata, pj.y, sp.nitems, patch,
                            reinterpret_cast<const float*>(sp.o.pfac), setab);
  }
}

template <int CC>
__global__ void __launch_bounds__(kThreads, 3) k_ragged_adj_reg_lp(const RaggedProb<float>* __restrict__ probs,
                                                                   const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<float> sp;
  __shared__ float2 setab[kLpEy + kLpEx];
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      if (threadIdx.x < kLpEy + kLpEx) setab[threadIdx.x] = probs[pj.x].etab[threadIdx.x];
      __syncthreads();
      cur = pj.x;
    }
    reg_job<CC, true>(sp.geo, sp.o, sp.tm, sp.ph, sp.kdata, sp.grid, sp.vec_ok, pj.y, smem_raw, nullptr, setab);
  }
}

// The exact passes of the linear-phase problems' left-out points, after the
// merged launches: blockIdx.y picks the problem (its index in lp_probs).
__global__ void __launch_bounds__(kThreads) k_ragged_fwd_fix(const RaggedProb<float>* __restrict__ probs,
                                                             const int* __restrict__ lp_probs) {
  const RaggedProb<float>& P = probs[lp_probs[blockIdx.y]];
  fwd_lp_fix_body(P.geo, P.a, P.tm, P.ph, P.grid, P.fix, P.nfix, P.kdata, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kThreads) k_ragged_adj_fix(const RaggedProb<float>* __restrict__ probs,
                                                             const int* __restrict__ lp_probs) {
  const RaggedProb<float>& P = probs[lp_probs[blockIdx.y]];
  adj_lp_fix_body(P.geo, P.o, P.tm, P.ph, P.kdata, P.fix, P.nfix, P.grid, blockIdx.x, gridDim.x);
}

template <typename R, int D, int JC>
__global__ void __launch_bounds__(kThreads) k_ragged_adj_own(const RaggedProb<R>* __restrict__ probs,
                                                             const int2* __restrict__ jobs, int64_t njobs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) RaggedProb<R> sp;
  int cur = -1;
  for (int64_t g = blockIdx.x; g < njobs; g += gridDim.x) {
    const int2 pj = jobs[g];
    if (pj.x != cur) {
      __syncthreads();
      load_desc(&sp, probs + pj.x);
      __syncthreads();
      cur = pj.x;
    }
    own_job<R, D, JC, false>(sp.geo, sp.o, sp.tm, sp.ph, sp.kdata, sp.grid, pj.y, smem_raw);
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
  int flags;  // the call's geometry flags (TKBN_TABLES_*, layout bits)
};

enum class Op { kFwd, kAdj, kGrad };

template <typename R>
static int prepare(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, int64_t B, int64_t C, Op op,
                   InterpPlan* ip) {
  int rc = points_layout(g, p, &ip->L);
  if (rc) return rc;
  ip->flags = g->flags;
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
  // (the 3D adjoint's register path takes at most 8 coils per job)
  const int cmax = g->dtype == TKBN_C64 ? ((op == Op::kAdj && g->ndim == 3) ? 8 : 16) : 8;
  a.Cc = next_pow2((int)(C < cmax ? C : cmax));
  a.ncc = (int)((C + a.Cc - 1) / a.Cc);
  a.nbpt = p->ntraj == 1 ? B : 1;
  int cells = 1;
  a.gtot = 1;
  bool j6 = true;
  for (int d = 0; d < g->ndim; ++d) {
    cells *= ip->L.tile[d] + g->numpoints[d] - 1;
    a.gtot *= g->grid_size[d];
    j6 = j6 && g->numpoints[d] == 6;
  }
  a.cells = cells;
  a.ps = cells | 1;  // odd plane stride spreads coil planes over banks
  const int nj = j6 ? 6 : kMaxJ;
  a.scratch = (32 / a.Cc) * g->ndim * nj;
  const size_t patch = op == Op::kAdj ? (size_t)2 * a.Cc * a.ps * sizeof(R) : (size_t)a.Cc * a.ps * sizeof(cplx<R>);
  // per-warp factor scratch: the table factors (the gradient keeps values and derivatives)
  ip->smem = patch + (size_t)kWarps * a.scratch * (op == Op::kGrad ? 2 : 1) * sizeof(cplx<R>);
  if (ip->smem > 220 * 1024)
    return set_error(TKBN_ERR_UNSUPPORTED, "tile patch needs %zu bytes of shared memory", ip->smem);
  ip->max_jobs = ip->L.max_items * a.nbpt * a.ncc;
  return TKBN_OK;
}

// Persistent grid: as many CTAs as are resident at once (no second wave), at
// most one per job.
template <typename K>
static int resident_blocks(K kernel, size_t smem, int64_t max_jobs, int* blocks) {
  int64_t b = 0;
  const int rc = resident_grid((const void*)kernel, kThreads, smem, &b);
  if (rc) return rc;
  if (max_jobs < b) b = max_jobs;
  *blocks = (int)(b < 1 ? 1 : b);
  return TKBN_OK;
}

// Calls fn(std::integral_constant<int, CC>) for CC in {2, 4, 8, 16}.
template <typename Fn>
static int with_cc(int CC, Fn&& fn) {
  switch (CC) {
    case 2: return fn(std::integral_constant<int, 2>{});
    case 4: return fn(std::integral_constant<int, 4>{});
    case 8: return fn(std::integral_constant<int, 8>{});
    default: return fn(std::integral_constant<int, 16>{});
  }
}

// The 2D per-point factor scratch of a layout (16 x 14 tiles, complex64,
// J = 6): per sorted point a record (16 floats in the linear-phase form, 12
// complex factors otherwise), then {Ey, Ex} and the left-out count past the
// records, the left-out list in the records' spare room.
struct PointFactors {
  float2* pf;
  float2* et;
  int32_t* fix;
  int32_t* nfix;
};

static PointFactors point_factors_of(const InterpPlan& ip, const char* ws) {
  PointFactors f;
  f.pf = (float2*)const_cast<char*>(ws + ip.L.off_pfac);
  f.et = f.pf + ip.a.n * 12;
  f.nfix = reinterpret_cast<int32_t*>(f.et + kLpEy + kLpEx + 8);
  f.fix = reinterpret_cast<int32_t*>(f.pf + ip.a.n * 8);
  return f;
}

// Whether the calls on this layout use the linear-phase factor records: the
// tables are linear-phase and the layout is not deterministic (the adjoint
// adds the left-out points with atomics).
static bool lp_factors(const InterpPlan& ip) {
  return ip.L.pfac && (ip.flags & TKBN_TABLES_LINEAR_PHASE) && !(ip.flags & TKBN_ADJ_DETERMINISTIC);
}

// 3D: whether the calls on this layout use the linear-phase records (the
// same conditions as in 2D).
static bool lp3_factors(const InterpPlan& ip) {
  return ip.L.pfac3 && (ip.flags & TKBN_TABLES_LINEAR_PHASE) && !(ip.flags & TKBN_ADJ_DETERMINISTIC);
}

// Fills the 3D records and the left-out list unless TKBN_ADJ_REUSE_FACTORS
// (an earlier call on this workspace left those of these tables and flags).
static int point_factors3_prepass(const Geo<float>& geo, const InterpPlan& ip, const char* ws, cudaStream_t s) {
  if (!lp3_factors(ip) || ip.a.n == 0 || (ip.flags & TKBN_ADJ_REUSE_FACTORS)) return TKBN_OK;
  int32_t* lfix = (int32_t*)const_cast<char*>(ws + ip.L.off_lfix);
  int rc = check_cuda(cudaMemsetAsync(lfix, 0, sizeof(int32_t), s), "reset left-out count");
  if (rc) return rc;
  const int64_t nb = (ip.a.n + kThreads - 1) / kThreads;
  k_point_factors3<<<(int)(nb < 152 * 16 ? nb : 152 * 16), kThreads, 0, s>>>(
      geo, (const float*)(ws + ip.L.off_coords), (const float2*)(ws + ip.L.off_phase), ip.a.n,
      (float*)const_cast<char*>(ws + ip.L.off_pfac3), lfix);
  return check_cuda(cudaGetLastError(), "point factor launch");
}

// Fills the factor scratch (lp: linear-phase records, else complex factors)
// unless the caller passed TKBN_ADJ_REUSE_FACTORS, vouching that an earlier
// call on this workspace left the factors of these tables and flags in place.
static int point_factors_prepass(const Geo<float>& geo, const InterpPlan& ip, const char* ws, bool lp,
                                 cudaStream_t s) {
  if (!ip.L.pfac || ip.a.n == 0 || (ip.flags & TKBN_ADJ_REUSE_FACTORS)) return TKBN_OK;
  const PointFactors f = point_factors_of(ip, ws);
  const int64_t nb = (2 * ip.a.n + kThreads - 1) / kThreads;
  const int grid_b = (int)(nb < 152 * 16 ? nb : 152 * 16);
  if (lp) {
    int rc = check_cuda(cudaMemsetAsync(f.nfix, 0, sizeof(int32_t), s), "reset left-out count");
    if (rc) return rc;
    k_point_factors2<true><<<grid_b, kThreads, 0, s>>>(geo, (const float*)(ws + ip.L.off_coords),
                                                        (const float2*)(ws + ip.L.off_phase), ip.a.n, f.pf, f.et,
                                                        f.fix, f.nfix);
  } else {
    k_point_factors2<false><<<grid_b, kThreads, 0, s>>>(geo, (const float*)(ws + ip.L.off_coords),
                                                         (const float2*)(ws + ip.L.off_phase), ip.a.n, f.pf, f.et,
                                                         f.fix, f.nfix);
  }
  return check_cuda(cudaGetLastError(), "point factor launch");
}

template <typename R, int D, int JC>
static int launch_fwd_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* grid, void* kdata,
                        cudaStream_t s) {
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    if (ip.a.Cc >= 2) {
      return with_cc(ip.a.Cc, [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        constexpr int PPW = 64 / CC;
        // linear-phase form: patches of at most kLpEy x kLpEx cells (the E tables' range)
        const bool lp = lp_factors(ip) && geo.P[0] <= kLpEy && geo.P[1] <= kLpEx;
        const size_t smem = (size_t)ip.a.cells * pair_cell_stride<CC>() * sizeof(float2) +
                            (size_t)kWarps * PPW * 2 * 6 * sizeof(float2) +
                            (lp ? (size_t)(kLpEy + kLpEx) * sizeof(float2) : 0);
        const float* tmp = (const float*)(ws + ip.L.off_coords);
        const float2* php = (const float2*)(ws + ip.L.off_phase);
        if (!lp) {
          int blocks;
          int rc = resident_blocks(k_interp_fwd_pairs<CC, false>, smem, ip.max_jobs, &blocks);
          if (rc) return rc;
          k_interp_fwd_pairs<CC, false><<<blocks, kThreads, smem, s>>>(geo, ip.a, tmp, php, (const float2*)grid,
                                                                       (float2*)kdata, nullptr);
          return check_cuda(cudaGetLastError(), "interp_fwd launch");
        }
        const PointFactors f = point_factors_of(ip, ws);
        int blocks;
        int rc = resident_blocks(k_interp_fwd_pairs<CC, true>, smem, ip.max_jobs, &blocks);
        if (rc) return rc;
        k_interp_fwd_pairs<CC, true><<<blocks, kThreads, smem, s>>>(geo, ip.a, tmp, php, (const float2*)grid,
                                                                    (float2*)kdata, (const float*)f.pf);
        rc = check_cuda(cudaGetLastError(), "interp_fwd launch");
        if (rc) return rc;
        k_fwd_lp_fix<<<152, kThreads, 0, s>>>(geo, ip.a, tmp, php, (const float2*)grid, f.fix, f.nfix,
                                              (float2*)kdata);
        return check_cuda(cudaGetLastError(), "interp_fwd fix launch");
      });
    }
  }
  if constexpr (std::is_same<R, float>::value && D == 3 && JC == 6) {
    // linear-phase tables on a 4 x 8 x 8 layout: real magnitudes from the
    // per-point records the pre-pass left (run by interp_fwd_r), up to 8 coils per job
    if (lp3_factors(ip) && geo.P[0] == kP3Z && geo.P[1] == kP3Y && geo.P[2] == kP3X) {
      Launch a3 = ip.a;
      a3.Cc = ip.a.C >= 8 ? 8 : next_pow2((int)ip.a.C);
      a3.ncc = (int)((ip.a.C + a3.Cc - 1) / a3.Cc);
      const int64_t max_jobs = ip.L.max_items * a3.nbpt * a3.ncc;
      const float* tmp = (const float*)(ws + ip.L.off_coords);
      const float* rec3 = (const float*)(ws + ip.L.off_pfac3);
      auto launch = [&](auto kernel, size_t smem) {
        int blocks;
        int rc2 = resident_blocks(kernel, smem, max_jobs, &blocks);
        if (rc2) return rc2;
        kernel<<<blocks, kThreads, smem, s>>>(geo, a3, tmp, (const float2*)grid, (float2*)kdata, rec3);
        return check_cuda(cudaGetLastError(), "interp_fwd launch");
      };
      int rc;
      switch (a3.Cc) {
        case 1: rc = launch(k_interp_fwd_lp3<1>, fwd_lp3_smem<1>()); break;
        case 2: rc = launch(k_interp_fwd_lp3<2>, fwd_lp3_smem<2>()); break;
        case 4: rc = launch(k_interp_fwd_lp3<4>, fwd_lp3_smem<4>()); break;
        default: rc = launch(k_interp_fwd_lp3<8>, fwd_lp3_smem<8>()); break;
      }
      if (rc) return rc;
      k_fwd_lp_fix3<<<152, kThreads, 0, s>>>(geo, a3, tmp, (const float2*)(ws + ip.L.off_phase),
                                             (const float2*)grid, (const int32_t*)(ws + ip.L.off_lfix),
                                             (float2*)kdata);
      return check_cuda(cudaGetLastError(), "interp_fwd fix launch");
    }
  }
  auto k = k_interp_fwd<R, D, JC>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords),
                                      (const cplx<R>*)(ws + ip.L.off_phase), (const cplx<R>*)grid, (cplx<R>*)kdata);
  return check_cuda(cudaGetLastError(), "interp_fwd launch");
}

template <typename R, int D, int JC>
static int launch_adj_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* kdata, void* grid,
                        cudaStream_t s) {
  auto k = k_interp_adj<R, D, JC>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords),
                                      (const cplx<R>*)(ws + ip.L.off_phase), (const cplx<R>*)kdata, (cplx<R>*)grid);
  return check_cuda(cudaGetLastError(), "interp_adj launch");
}

template <typename R, int D, int JC>
static int launch_grad_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* grid, const void* v,
                         void* grad, cudaStream_t s) {
  auto k = k_interp_grad<R, D, JC>;
  int blocks;
  int rc = resident_blocks(k, ip.smem, ip.max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, ip.smem, s>>>(geo, ip.a, (const R*)(ws + ip.L.off_coords),
                                      (const cplx<R>*)(ws + ip.L.off_phase), (const cplx<R>*)grid,
                                      (const cplx<R>*)v, (R*)grad);
  return check_cuda(cudaGetLastError(), "interp_grad launch");
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
  int rc = prepare<R>(g, p, ws, B, C, Op::kFwd, &ip);
  if (rc) return rc;
  if (p->npts == 0) return TKBN_OK;
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, nullptr);
  const char* w = (const char*)ws;
  if constexpr (std::is_same<R, float>::value) {
    // every forward or adjoint call on a layout with a factor scratch leaves
    // the factors of its tables and flags there, whichever kernel it runs
    if (ip.L.pfac && (rc = point_factors_prepass(geo, ip, w, lp_factors(ip), s))) return rc;
    if (ip.L.pfac3 && (rc = point_factors3_prepass(geo, ip, w, s))) return rc;
  }
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

template <int D>
constexpr int max_combo() {
  return D == 1 ? 8 : (D == 2 ? 16 : 27);
}

// Tensor map of a complex64 grid (planes x K0 x K1) as floats, box = one
// 16 x 14 tile of `planes_box` planes, for the register adjoint's tensor
// stores. False when the driver entry point is missing or encoding fails
// (the kernel then writes rows itself).
static bool grid_tensor_map(void* grid, int64_t K0, int64_t K1, int64_t planes, int planes_box, CUtensorMap* out) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }();
  if (!encode || (uintptr_t)grid % 16 != 0 || K1 % 2 != 0 || planes < 1) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)(2 * K1), (cuuint64_t)K0, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)(2 * K1 * 4), (cuuint64_t)(K0 * K1 * 8)};
  const cuuint32_t box[3] = {2 * kRegTileX, kRegTileY, (cuuint32_t)planes_box};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, grid, dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static OwnLaunch make_own(const InterpPlan& ip, const char* ws, int D) {
  OwnLaunch o;
  o.jobs = (const Item*)(ws + ip.L.off_adj_jobs);
  o.hdr = ip.a.hdr;
  o.counts = (const int32_t*)(ws + ip.L.off_counts);
  o.tile_off = (const int32_t*)(ws + ip.L.off_tile_off);
  o.vals = ip.a.vals;
  o.n = ip.a.n;
  o.M = ip.a.M;
  o.ntraj = ip.a.ntraj;
  o.B = ip.a.B;
  o.C = ip.a.C;
  o.Cc = ip.a.Cc;
  o.ncc = ip.a.ncc;
  o.nbpt = ip.a.nbpt;
  int tcells = 1;
  for (int d = 0; d < D; ++d) tcells *= ip.L.tile[d];
  o.aps = tcells | 1;
  o.gtot = ip.a.gtot;
  o.span = ip.L.span;
  o.vlist = ip.L.vlist ? (const int4*)(ws + ip.L.off_vlist) : nullptr;
  o.voff = ip.L.vlist ? (const int32_t*)(ws + ip.L.off_voff) : nullptr;
  o.koff = (ip.L.ksort || ip.L.csort) ? (const int32_t*)(ws + ip.L.off_koff) : nullptr;
  o.pfac = nullptr;  // set by the launch that fills it
  o.vsort = ip.L.csort ? (const int4*)(ws + ip.L.off_vsort) : nullptr;
  return o;
}

// Shared memory of the generic owned-tile adjoint for Cc coils per job.
template <typename R, int D, int JC>
static size_t own_smem(const OwnLaunch& o) {
  constexpr int NJ = NJOf<JC>::N;
  return (size_t)o.Cc * o.aps * sizeof(cplx<R>) + (size_t)kNB * D * NJ * sizeof(cplx<R>) +
         (size_t)kNB * o.Cc * sizeof(cplx<R>) +
         sizeof(int) * ((size_t)kNB * D + kNB + 2 * max_combo<D>() + 1 + kNB / 32);
}

// The register adjoint applies: 2D complex64, J = 6, 16 x 14 tiles with
// per-tile point lists (any coil count; CC = max(2, coils per job)).
template <typename R, int D, int JC>
static bool reg_eligible(const InterpPlan& ip, const OwnLaunch& o) {
  return std::is_same<R, float>::value && D == 2 && JC == 6 && o.vlist && o.vsort && o.koff && o.Cc <= kRegCoils &&
         ip.L.tile[0] == kRegTileY && ip.L.tile[1] == kRegTileX && ip.L.knk == kRegKeys;
}

static int reg_cc(int Cc) { return Cc < 2 ? 2 : Cc; }

// Staging of a batch, or (more than one point group) the groups' partial tiles.
// 3D: 4 x 8 x 8 tiles, at most 8 coils per job.
template <typename R, int D, int JC>
static bool reg3_eligible(const InterpPlan& ip, const OwnLaunch& o) {
  return std::is_same<R, float>::value && D == 3 && JC == 6 && o.vlist && o.vsort && o.koff && o.Cc <= 8 &&
         ip.L.tile[0] == kReg3Z && ip.L.tile[1] == kReg3Y && ip.L.tile[2] == kReg3X && ip.L.knk == kReg3Keys;
}

static size_t reg3_smem(int CC) {
  const size_t staging = reg3_etab_offset(CC) + (size_t)3 * kLp3En * sizeof(float2);
  const int ng = kWarps / (kReg3Rows / (32 / CC));
  const size_t partials = ng > 1 ? (size_t)ng * kReg3Rows * kReg3X * CC * sizeof(float2) : 0;
  return staging > partials ? staging : partials;
}

static size_t reg_smem(int CC) {
  const size_t staging = reg_rtab_offset(CC) + (size_t)(kLpEy + kLpEx) * sizeof(float2);
  const int ng = kWarps / (kRegTileY / (32 / CC));
  const size_t partials = ng > 1 ? (size_t)ng * kRegTileY * kRegTileX * CC * sizeof(float2) : 0;
  return staging > partials ? staging : partials;
}

template <typename R, int D, int JC>
static int launch_adj_own_t(const Geo<R>& geo, const InterpPlan& ip, const char* ws, const void* kdata, void* grid,
                            cudaStream_t s) {
  const OwnLaunch o = make_own(ip, ws, D);
  const size_t smem = own_smem<R, D, JC>(o);
  if (smem > 220 * 1024) return set_error(TKBN_ERR_UNSUPPORTED, "adjoint tile needs %zu bytes of shared memory", smem);
  const int64_t max_jobs = ip.L.max_subjobs * o.nbpt * o.ncc;
  // split tiles are accumulated atomically: zero them first. Blocks
  // (x, y) take the split tiles x, x + gridDim.x, ... and within each the
  // rows y*8 + warp, strided by 8*gridDim.y.
  {
    const int64_t zx = ip.L.max_subjobs < 152 ? ip.L.max_subjobs : 152;
    k_zero_split_tiles<R, D><<<dim3((unsigned)(zx < 1 ? 1 : zx), 16), 256, 0, s>>>(geo, o, ip.L.adj_chunk,
                                                                                  (cplx<R>*)grid);
    int rc = check_cuda(cudaGetLastError(), "zero split tiles launch");
    if (rc) return rc;
  }
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    if (reg_eligible<R, D, JC>(ip, o)) {
      OwnLaunch orr = o;
      // linear-phase tables: real factors (needs the per-point pre-pass)
      // (a deterministic layout keeps the table path: the linear-phase form
      // adds its left-out points with atomics)
      // the factor scratch was filled (or vouched for) by interp_adj_r
      const bool lp = lp_factors(ip);
      const PointFactors f = point_factors_of(ip, ws);
      float2* pf = f.pf;
      int32_t* nfix = f.nfix;
      int32_t* fix = f.fix;
      if (ip.L.pfac && ip.a.n > 0) orr.pfac = pf;
      return with_cc(reg_cc(o.Cc), [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        const size_t rsmem = reg_smem(CC);
        const int vec_ok = ((uintptr_t)grid % 16 == 0) && (geo.K[1] % 2 == 0);
        CUtensorMap tmap;
        std::memset(&tmap, 0, sizeof(tmap));
        const int use_tmap = CC == kRegCoils && vec_ok && grid_tensor_map(grid, geo.K[0], geo.K[1], o.B * o.C, CC, &tmap);
        auto launch = [&](auto kernel) {
          int blocks;
          int rc = resident_blocks(kernel, rsmem, max_jobs, &blocks);
          if (rc) return rc;
          kernel<<<blocks, kThreads, rsmem, s>>>(geo, orr, (const float*)(ws + ip.L.off_coords),
                                                 (const float2*)(ws + ip.L.off_phase), (const float2*)kdata,
                                                 (float2*)grid, vec_ok, use_tmap, tmap);
          return check_cuda(cudaGetLastError(), "interp_adj launch");
        };
        if (!(lp && orr.pfac)) return launch(k_interp_adj_reg<CC, false>);
        int rc = launch(k_interp_adj_reg<CC, true>);
        if (rc) return rc;
        k_adj_lp_fix<<<152, kThreads, 0, s>>>(geo, orr, (const float*)(ws + ip.L.off_coords),
                                               (const float2*)(ws + ip.L.off_phase), (const float2*)kdata, fix, nfix,
                                               (float2*)grid);
        return check_cuda(cudaGetLastError(), "interp_adj fix launch");
      });
    }
  }
  if constexpr (std::is_same<R, float>::value && D == 3 && JC == 6) {
    if (reg3_eligible<R, D, JC>(ip, o)) {
      return with_cc(reg_cc(o.Cc), [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value < 8 ? decltype(ccv)::value : 8;
        const size_t rsmem = reg3_smem(CC);
        const int vec_ok = ((uintptr_t)grid % 16 == 0) && (geo.K[2] % 2 == 0);
        // linear-phase tables: real kernel values (not for deterministic layouts:
        // the left-out points are added with atomics)
        // (the records and the left-out list come from the pre-pass, run by interp_adj_r)
        const bool lp = lp3_factors(ip);
        int32_t* lfix = lp ? (int32_t*)const_cast<char*>(ws + ip.L.off_lfix) : nullptr;
        const float* rec3 = lp ? (const float*)(ws + ip.L.off_pfac3) : nullptr;
        auto launch = [&](auto kernel) {
          int blocks;
          int rc = resident_blocks(kernel, rsmem, max_jobs, &blocks);
          if (rc) return rc;
          kernel<<<blocks, kThreads, rsmem, s>>>(geo, o, (const float*)(ws + ip.L.off_coords),
                                                 (const float2*)(ws + ip.L.off_phase), (const float2*)kdata,
                                                 (float2*)grid, vec_ok, rec3);
          return check_cuda(cudaGetLastError(), "interp_adj launch");
        };
        if (!lp) return launch(k_interp_adj_reg3<CC, false>);
        int rc = launch(k_interp_adj_reg3<CC, true>);
        if (rc) return rc;
        k_adj_lp_fix3<<<152, kThreads, 0, s>>>(geo, o, (const float*)(ws + ip.L.off_coords),
                                                (const float2*)(ws + ip.L.off_phase), (const float2*)kdata, lfix,
                                                (float2*)grid);
        return check_cuda(cudaGetLastError(), "interp_adj fix launch");
      });
    }
  }
  const bool fast = D == 2 && JC == 6 && o.Cc == 16 && ip.L.tile[0] == 2 * kWarps;
  auto k = fast ? k_interp_adj_own<R, D, JC, true> : k_interp_adj_own<R, D, JC, false>;
  int blocks;
  int rc = resident_blocks(k, smem, max_jobs, &blocks);
  if (rc) return rc;
  k<<<blocks, kThreads, smem, s>>>(geo, o, (const R*)(ws + ip.L.off_coords), (const cplx<R>*)(ws + ip.L.off_phase),
                                   (const cplx<R>*)kdata, (cplx<R>*)grid);
  return check_cuda(cudaGetLastError(), "interp_adj launch");
}

template <typename R, int D, int JC>
static int adj_dispatch(const Geo<R>& geo, const InterpPlan& ip, const char* w, const void* kdata, void* grid,
                        int64_t B, int64_t C, cudaStream_t s) {
  if (ip.L.owned_ok && ip.L.span.ncombo <= max_combo<D>()) return launch_adj_own_t<R, D, JC>(geo, ip, w, kdata, grid, s);
  int rc = check_cuda(cudaMemsetAsync(grid, 0, (size_t)(B * C * ip.a.gtot) * sizeof(cplx<R>), s), "zero grid");
  if (rc) return rc;
  return launch_adj_t<R, D, JC>(geo, ip, w, kdata, grid, s);
}

template <typename R>
static int interp_adj_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                        const void* kdata, int64_t B, int64_t C, void* grid, cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, Op::kAdj, &ip);
  if (rc) return rc;
  if (p->npts == 0)
    return check_cuda(cudaMemsetAsync(grid, 0, (size_t)(B * C * ip.a.gtot) * sizeof(cplx<R>), s), "zero grid");
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, nullptr);
  const char* w = (const char*)ws;
  if constexpr (std::is_same<R, float>::value) {
    // every forward or adjoint call on a layout with a factor scratch leaves
    // the factors of its tables and flags there, whichever kernel it runs
    if (ip.L.pfac && (rc = point_factors_prepass(geo, ip, w, lp_factors(ip), s))) return rc;
    if (ip.L.pfac3 && (rc = point_factors3_prepass(geo, ip, w, s))) return rc;
  }
  const bool j6 = all_j(g, 6);
  switch (g->ndim) {
    case 1:
      return j6 ? adj_dispatch<R, 1, 6>(geo, ip, w, kdata, grid, B, C, s)
                : adj_dispatch<R, 1, 0>(geo, ip, w, kdata, grid, B, C, s);
    case 2:
      return j6 ? adj_dispatch<R, 2, 6>(geo, ip, w, kdata, grid, B, C, s)
                : adj_dispatch<R, 2, 0>(geo, ip, w, kdata, grid, B, C, s);
    default:
      return j6 ? adj_dispatch<R, 3, 6>(geo, ip, w, kdata, grid, B, C, s)
                : adj_dispatch<R, 3, 0>(geo, ip, w, kdata, grid, B, C, s);
  }
}

template <typename R>
static int interp_adj_atomic_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws,
                               const void* const* tables, const void* kdata, int64_t B, int64_t C, void* grid,
                               cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, Op::kAdj, &ip);
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

template <typename R>
static int interp_grad_r(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
                         const void* const* dtables, const void* grid, const void* v, int64_t B, int64_t C,
                         void* grad, cudaStream_t s) {
  InterpPlan ip;
  int rc = prepare<R>(g, p, ws, B, C, Op::kGrad, &ip);
  if (rc) return rc;
  if (!dtables) return set_error(TKBN_ERR_INVALID, "derivative tables are required");
  rc = check_cuda(cudaMemsetAsync(grad, 0, (size_t)(p->ntraj * g->ndim * p->npts) * sizeof(R), s), "zero grad");
  if (rc || p->npts == 0) return rc;
  Geo<R> geo = make_geo<R>(g, &ip.L, tables, dtables);
  const char* w = (const char*)ws;
  const bool j6 = all_j(g, 6);
  switch (g->ndim) {
    case 1:
      return j6 ? launch_grad_t<R, 1, 6>(geo, ip, w, grid, v, grad, s) : launch_grad_t<R, 1, 0>(geo, ip, w, grid, v, grad, s);
    case 2:
      return j6 ? launch_grad_t<R, 2, 6>(geo, ip, w, grid, v, grad, s) : launch_grad_t<R, 2, 0>(geo, ip, w, grid, v, grad, s);
    default:
      return j6 ? launch_grad_t<R, 3, 6>(geo, ip, w, grid, v, grad, s) : launch_grad_t<R, 3, 0>(geo, ip, w, grid, v, grad, s);
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

// ---------------------------------------------------------------- K8 ragged plan

}  // namespace tkbn_host

struct tkbn_ragged_plan_s {
  int dtype, ndim, j6;
  int64_t nprob;
  void* probs;  // RaggedProb<R>[nprob] on the device
  // fwd_pairs[k], reg_jobs[k]: jobs of problems with 2 << k coils per job
  // (the _lp lists: linear-phase problems)
  int2 *fwd_jobs, *fwd_pairs[4], *reg_jobs[4], *own_jobs, *zero_jobs;
  int2 *fwd_pairs_lp[4], *reg_jobs_lp[4];
  int64_t n_fwd, n_fwd_pairs[4], n_reg[4], n_own, n_zero, n_fwd_pairs_lp[4], n_reg_lp[4];
  size_t smem_fwd, smem_fwd_pairs[4], smem_own;
  int* lp_probs;  // the linear-phase problems, for the exact passes
  int64_t n_lp;
};

namespace tkbn_host {

namespace {

struct JobRec {
  int len;
  int p;
  int j;
};

// Longest first, then problem and job index (a fixed order).
void lpt_sort(std::vector<JobRec>& v) {
  std::stable_sort(v.begin(), v.end(), [](const JobRec& x, const JobRec& y) { return x.len > y.len; });
}

int upload_jobs(const std::vector<JobRec>& v, int2** dev) {
  *dev = nullptr;
  if (v.empty()) return TKBN_OK;
  std::vector<int2> h(v.size());
  for (size_t i = 0; i < v.size(); ++i) h[i] = make_int2(v[i].p, v[i].j);
  int rc = check_cuda(cudaMalloc((void**)dev, h.size() * sizeof(int2)), "ragged job list");
  if (rc) return rc;
  return check_cuda(cudaMemcpy(*dev, h.data(), h.size() * sizeof(int2), cudaMemcpyHostToDevice), "ragged job upload");
}

template <typename R, int D, int JC>
int ragged_build(const tkbn_ragged_problem* pr, int64_t n, tkbn_ragged_plan_s* P) {
  std::vector<RaggedProb<R>> desc((size_t)n);
  std::vector<JobRec> fwd, fwdp[4], reg[4], own, zero, fwdp_lp[4], reg_lp[4];
  std::vector<int> lp_list;
  P->smem_fwd = 0;
  P->smem_own = 0;
  for (int k = 0; k < 4; ++k) P->smem_fwd_pairs[k] = 0;
  for (int64_t q = 0; q < n; ++q) {
    const tkbn_ragged_problem& r = pr[q];
    InterpPlan ip;
    int rc = prepare<R>(&r.geom, &r.points, r.workspace, 1, r.ncoil, Op::kFwd, &ip);
    if (rc) return rc;
    if (!r.grid || !r.kdata) return set_error(TKBN_ERR_INVALID, "problem %lld: null grid or kdata", (long long)q);
    const char* ws = (const char*)r.workspace;
    int64_t hdr[2] = {0, 0};
    if ((rc = check_cuda(cudaMemcpy(hdr, ip.a.hdr, sizeof(hdr), cudaMemcpyDeviceToHost), "read layout header")))
      return rc;
    RaggedProb<R>& d = desc[(size_t)q];
    memset(&d, 0, sizeof(d));
    d.geo = make_geo<R>(&r.geom, &ip.L, r.tables, nullptr);
    d.a = ip.a;
    d.o = make_own(ip, ws, D);
    d.tm = (const R*)(ws + ip.L.off_coords);
    d.ph = (const cplx<R>*)(ws + ip.L.off_phase);
    d.grid = (cplx<R>*)r.grid;
    d.kdata = (cplx<R>*)r.kdata;
    d.nitems = hdr[0];
    d.vec_ok = ((uintptr_t)r.grid % 16 == 0) && (r.geom.grid_size[D - 1] % 2 == 0);
    // linear-phase problems (16 x 14 register-adjoint layouts, linear-phase
    // tables, not deterministic) run both directions in the real form
    bool lpq = false;
    if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6)
      lpq = lp_factors(ip) && ip.a.n > 0 && reg_eligible<R, D, JC>(ip, make_own(ip, ws, D));
    // forward jobs: item i % nitems of coil chunk i / nitems; 2D complex64
    // J = 6 problems with 2 or more coils per job take the coil-pair gather
    const bool pairs = std::is_same<R, float>::value && D == 2 && JC == 6 && ip.a.Cc >= 2;
    const int pk = ip.a.Cc == 2 ? 0 : (ip.a.Cc == 4 ? 1 : (ip.a.Cc == 8 ? 2 : 3));
    if (pairs) {
      const int cc = 2 << pk;  // the kernel's coils per job
      const size_t sm = (size_t)ip.a.cells * (cc + 2) * sizeof(float2) + (size_t)kWarps * (64 / cc) * 12 * sizeof(float2);
      if (sm > P->smem_fwd_pairs[pk]) P->smem_fwd_pairs[pk] = sm;
    } else if (ip.smem > P->smem_fwd) {
      P->smem_fwd = ip.smem;
    }
    if (r.points.npts > 0 && hdr[0] > 0) {
      std::vector<Item> items((size_t)hdr[0]);
      if ((rc = check_cuda(cudaMemcpy(items.data(), ip.a.items, items.size() * sizeof(Item), cudaMemcpyDeviceToHost),
                           "read work items")))
        return rc;
      for (int64_t j = 0; j < hdr[0] * ip.a.ncc; ++j)
        (pairs ? (lpq ? fwdp_lp[pk] : fwdp[pk]) : fwd).push_back({items[(size_t)(j % hdr[0])].len, (int)q, (int)j});
    }
    // adjoint jobs: sub-job j / ncc of coil chunk j % ncc
    if (!ip.L.owned_ok || ip.L.span.ncombo > max_combo<D>())
      return set_error(TKBN_ERR_UNSUPPORTED, "problem %lld: grid too small for the owned-tile adjoint", (long long)q);
    std::vector<Item> sj((size_t)hdr[1]);
    if (hdr[1] > 0 &&
        (rc = check_cuda(cudaMemcpy(sj.data(), d.o.jobs, sj.size() * sizeof(Item), cudaMemcpyDeviceToHost),
                         "read adjoint sub-jobs")))
      return rc;
    const bool use_reg = reg_eligible<R, D, JC>(ip, d.o);
    if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
      if (use_reg && ip.L.pfac && ip.a.n > 0) {
        // the plan's trajectories and tables are fixed: the register adjoint's
        // per-point factors (linear-phase records, with the E tables and the
        // left-out list, for lp problems) are computed once, into the problem's workspace
        const PointFactors f = point_factors_of(ip, ws);
        const int64_t nb = (2 * ip.a.n + kThreads - 1) / kThreads;
        const int gb = (int)(nb < 152 * 16 ? nb : 152 * 16);
        if (lpq) {
          if ((rc = check_cuda(cudaMemset(f.nfix, 0, sizeof(int32_t)), "reset left-out count"))) return rc;
          k_point_factors2<true><<<gb, kThreads>>>(d.geo, d.tm, d.ph, ip.a.n, f.pf, f.et, f.fix, f.nfix);
          d.lp = 1;
          d.etab = f.et;
          d.fix = f.fix;
          d.nfix = f.nfix;
          lp_list.push_back((int)q);
        } else {
          k_point_factors2<false><<<gb, kThreads>>>(d.geo, d.tm, d.ph, ip.a.n, f.pf, nullptr, nullptr, nullptr);
        }
        if ((rc = check_cuda(cudaGetLastError(), "ragged factor pre-pass"))) return rc;
        d.o.pfac = f.pf;
      }
    }
    if (!use_reg) {
      const size_t sm = own_smem<R, D, JC>(d.o);
      if (sm > 220 * 1024) return set_error(TKBN_ERR_UNSUPPORTED, "adjoint tile needs %zu bytes of shared memory", sm);
      if (sm > P->smem_own) P->smem_own = sm;
    }
    const int rk = reg_cc(d.o.Cc) == 2 ? 0 : (reg_cc(d.o.Cc) == 4 ? 1 : (reg_cc(d.o.Cc) == 8 ? 2 : 3));
    for (int64_t j = 0; j < hdr[1] * ip.a.ncc; ++j) {
      const Item& it = sj[(size_t)(j / ip.a.ncc)];
      (use_reg ? (lpq ? reg_lp[rk] : reg[rk]) : own).push_back({it.len, (int)q, (int)j});
    }
    for (int64_t j = 0; j < hdr[1]; ++j)
      if (sj[(size_t)j].pad && sj[(size_t)j].start == 0) zero.push_back({sj[(size_t)j].len, (int)q, (int)j});
  }
  // the factor pre-passes (legacy stream) end before the plan is returned
  if (int rc = check_cuda(cudaStreamSynchronize(0), "ragged factor pre-pass")) return rc;
  lpt_sort(fwd);
  for (auto& v : fwdp) lpt_sort(v);
  for (auto& v : reg) lpt_sort(v);
  for (auto& v : fwdp_lp) lpt_sort(v);
  for (auto& v : reg_lp) lpt_sort(v);
  lpt_sort(own);
  int rc = check_cuda(cudaMalloc(&P->probs, desc.size() * sizeof(RaggedProb<R>)), "ragged descriptors");
  if (rc) return rc;
  if ((rc = check_cuda(cudaMemcpy(P->probs, desc.data(), desc.size() * sizeof(RaggedProb<R>), cudaMemcpyHostToDevice),
                       "ragged descriptor upload")))
    return rc;
  if ((rc = upload_jobs(fwd, &P->fwd_jobs)) || (rc = upload_jobs(own, &P->own_jobs)) ||
      (rc = upload_jobs(zero, &P->zero_jobs)))
    return rc;
  for (int k = 0; k < 4; ++k) {
    if ((rc = upload_jobs(reg[k], &P->reg_jobs[k]))) return rc;
    if ((rc = upload_jobs(fwdp[k], &P->fwd_pairs[k]))) return rc;
    if ((rc = upload_jobs(reg_lp[k], &P->reg_jobs_lp[k]))) return rc;
    if ((rc = upload_jobs(fwdp_lp[k], &P->fwd_pairs_lp[k]))) return rc;
    P->n_reg[k] = (int64_t)reg[k].size();
    P->n_fwd_pairs[k] = (int64_t)fwdp[k].size();
    P->n_reg_lp[k] = (int64_t)reg_lp[k].size();
    P->n_fwd_pairs_lp[k] = (int64_t)fwdp_lp[k].size();
  }
  P->n_lp = (int64_t)lp_list.size();
  P->lp_probs = nullptr;
  if (P->n_lp > 0) {
    if ((rc = check_cuda(cudaMalloc((void**)&P->lp_probs, lp_list.size() * sizeof(int)), "ragged lp list"))) return rc;
    if ((rc = check_cuda(cudaMemcpy(P->lp_probs, lp_list.data(), lp_list.size() * sizeof(int), cudaMemcpyHostToDevice),
                         "ragged lp list upload")))
      return rc;
  }
  P->n_fwd = (int64_t)fwd.size();
  P->n_own = (int64_t)own.size();
  P->n_zero = (int64_t)zero.size();
  return TKBN_OK;
}

template <typename R, int D, int JC>
int ragged_fwd_t(const tkbn_ragged_plan_s* P, cudaStream_t s) {
  int rc;
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    for (int k = 0; k < 4; ++k) {
      if (P->n_fwd_pairs[k] == 0) continue;
      rc = with_cc(2 << k, [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        int blocks;
        int r = resident_blocks(k_ragged_fwd_pairs<CC>, P->smem_fwd_pairs[k], P->n_fwd_pairs[k], &blocks);
        if (r) return r;
        k_ragged_fwd_pairs<CC><<<blocks, kThreads, P->smem_fwd_pairs[k], s>>>(
            (const RaggedProb<float>*)P->probs, P->fwd_pairs[k], P->n_fwd_pairs[k]);
        return check_cuda(cudaGetLastError(), "ragged interp_fwd launch");
      });
      if (rc) return rc;
    }
    for (int k = 0; k < 4; ++k) {
      if (P->n_fwd_pairs_lp[k] == 0) continue;
      rc = with_cc(2 << k, [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        int blocks;
        int r = resident_blocks(k_ragged_fwd_pairs_lp<CC>, P->smem_fwd_pairs[k], P->n_fwd_pairs_lp[k], &blocks);
        if (r) return r;
        k_ragged_fwd_pairs_lp<CC><<<blocks, kThreads, P->smem_fwd_pairs[k], s>>>(
            (const RaggedProb<float>*)P->probs, P->fwd_pairs_lp[k], P->n_fwd_pairs_lp[k]);
        return check_cuda(cudaGetLastError(), "ragged interp_fwd launch");
      });
      if (rc) return rc;
    }
  }
  if (P->n_fwd > 0) {
    int blocks;
    rc = resident_blocks(k_ragged_fwd<R, D, JC>, P->smem_fwd, P->n_fwd, &blocks);
    if (rc) return rc;
    k_ragged_fwd<R, D, JC><<<blocks, kThreads, P->smem_fwd, s>>>((const RaggedProb<R>*)P->probs, P->fwd_jobs,
                                                                 P->n_fwd);
    if ((rc = check_cuda(cudaGetLastError(), "ragged interp_fwd launch"))) return rc;
  }
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    if (P->n_lp > 0) {
      k_ragged_fwd_fix<<<dim3(16, (unsigned)P->n_lp), kThreads, 0, s>>>((const RaggedProb<float>*)P->probs,
                                                                          P->lp_probs);
      return check_cuda(cudaGetLastError(), "ragged interp_fwd fix launch");
    }
  }
  return TKBN_OK;
}

template <typename R, int D, int JC>
int ragged_adj_t(const tkbn_ragged_plan_s* P, cudaStream_t s) {
  int rc;
  const RaggedProb<R>* probs = (const RaggedProb<R>*)P->probs;
  if (P->n_zero > 0) {
    const int64_t zx = P->n_zero < 152 ? P->n_zero : 152;
    k_ragged_zero<R, D><<<dim3((unsigned)zx, 16), 256, 0, s>>>(probs, P->zero_jobs, P->n_zero);
    if ((rc = check_cuda(cudaGetLastError(), "ragged zero launch"))) return rc;
  }
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    for (int k = 0; k < 4; ++k) {
      if (P->n_reg[k] == 0) continue;
      rc = with_cc(2 << k, [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        int blocks;
        int r = resident_blocks(k_ragged_adj_reg<CC>, reg_smem(CC), P->n_reg[k], &blocks);
        if (r) return r;
        k_ragged_adj_reg<CC><<<blocks, kThreads, reg_smem(CC), s>>>(probs, P->reg_jobs[k], P->n_reg[k]);
        return check_cuda(cudaGetLastError(), "ragged interp_adj launch");
      });
      if (rc) return rc;
    }
    for (int k = 0; k < 4; ++k) {
      if (P->n_reg_lp[k] == 0) continue;
      rc = with_cc(2 << k, [&](auto ccv) {
        constexpr int CC = decltype(ccv)::value;
        int blocks;
        int r = resident_blocks(k_ragged_adj_reg_lp<CC>, reg_smem(CC), P->n_reg_lp[k], &blocks);
        if (r) return r;
        k_ragged_adj_reg_lp<CC><<<blocks, kThreads, reg_smem(CC), s>>>(probs, P->reg_jobs_lp[k], P->n_reg_lp[k]);
        return check_cuda(cudaGetLastError(), "ragged interp_adj launch");
      });
      if (rc) return rc;
    }
  }
  if (P->n_own > 0) {
    int blocks;
    if ((rc = resident_blocks(k_ragged_adj_own<R, D, JC>, P->smem_own, P->n_own, &blocks))) return rc;
    k_ragged_adj_own<R, D, JC><<<blocks, kThreads, P->smem_own, s>>>(probs, P->own_jobs, P->n_own);
    if ((rc = check_cuda(cudaGetLastError(), "ragged interp_adj launch"))) return rc;
  }
  if constexpr (std::is_same<R, float>::value && D == 2 && JC == 6) {
    // the left-out points' exact contributions, after every tile is written
    if (P->n_lp > 0) {
      k_ragged_adj_fix<<<dim3(16, (unsigned)P->n_lp), kThreads, 0, s>>>((const RaggedProb<float>*)P->probs,
                                                                          P->lp_probs);
      return check_cuda(cudaGetLastError(), "ragged interp_adj fix launch");
    }
  }
  return TKBN_OK;
}

// Calls fn.template operator()<R, D, JC>() for the plan's dtype, ndim and numpoints.
template <typename Fn>
int ragged_dispatch(int dtype, int ndim, int j6, Fn&& fn) {
  auto by_d = [&](auto r) -> int {
    using R = decltype(r);
    switch (ndim) {
      case 1: return j6 ? fn.template run<R, 1, 6>() : fn.template run<R, 1, 0>();
      case 2: return j6 ? fn.template run<R, 2, 6>() : fn.template run<R, 2, 0>();
      default: return j6 ? fn.template run<R, 3, 6>() : fn.template run<R, 3, 0>();
    }
  };
  return dtype == TKBN_C64 ? by_d(float{}) : by_d(double{});
}

struct BuildFn {
  const tkbn_ragged_problem* pr;
  int64_t n;
  tkbn_ragged_plan_s* P;
  template <typename R, int D, int JC>
  int run() const { return ragged_build<R, D, JC>(pr, n, P); }
};
struct FwdFn {
  const tkbn_ragged_plan_s* P;
  cudaStream_t s;
  template <typename R, int D, int JC>
  int run() const { return ragged_fwd_t<R, D, JC>(P, s); }
};
struct AdjFn {
  const tkbn_ragged_plan_s* P;
  cudaStream_t s;
  template <typename R, int D, int JC>
  int run() const { return ragged_adj_t<R, D, JC>(P, s); }
};

}  // namespace

int ragged_plan_destroy(tkbn_ragged_plan p) {
  if (!p) return TKBN_OK;
  cudaFree(p->probs);
  cudaFree(p->fwd_jobs);
  for (int k = 0; k < 4; ++k) {
    cudaFree(p->reg_jobs[k]);
    cudaFree(p->fwd_pairs[k]);
    cudaFree(p->reg_jobs_lp[k]);
    cudaFree(p->fwd_pairs_lp[k]);
  }
  cudaFree(p->lp_probs);
  cudaFree(p->own_jobs);
  cudaFree(p->zero_jobs);
  delete p;
  return check_cuda(cudaGetLastError(), "ragged plan free");
}

int ragged_plan_create(const tkbn_ragged_problem* pr, int64_t n, tkbn_ragged_plan* out) {
  if (!pr || !out || n < 1) return set_error(TKBN_ERR_INVALID, "need at least one problem");
  const tkbn_geometry& g0 = pr[0].geom;
  if (g0.dtype != TKBN_C64 && g0.dtype != TKBN_C128) return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype");
  if (g0.ndim < 1 || g0.ndim > 3) return set_error(TKBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3");
  const int j6 = all_j(&g0, 6) ? 1 : 0;
  for (int64_t q = 0; q < n; ++q) {
    const tkbn_geometry& g = pr[q].geom;
    if (g.dtype != g0.dtype || g.ndim != g0.ndim || (all_j(&g, 6) ? 1 : 0) != j6)
      return set_error(TKBN_ERR_INVALID, "problem %lld: all problems need the same dtype, ndim and numpoints",
                       (long long)q);
    if (pr[q].points.ntraj != 1) return set_error(TKBN_ERR_INVALID, "problem %lld: ntraj must be 1", (long long)q);
    if (pr[q].ncoil < 1) return set_error(TKBN_ERR_INVALID, "problem %lld: ncoil must be >= 1", (long long)q);
  }
  tkbn_ragged_plan_s* P = new (std::nothrow) tkbn_ragged_plan_s();
  if (!P) return set_error(TKBN_ERR_INVALID, "out of host memory");
  P->dtype = g0.dtype;
  P->ndim = g0.ndim;
  P->j6 = j6;
  P->nprob = n;
  const int rc = ragged_dispatch(P->dtype, P->ndim, j6, BuildFn{pr, n, P});
  if (rc) {
    ragged_plan_destroy(P);
    return rc;
  }
  *out = P;
  return TKBN_OK;
}

int ragged_interp_fwd(tkbn_ragged_plan p, cudaStream_t s) {
  if (!p) return set_error(TKBN_ERR_INVALID, "ragged plan is null");
  return ragged_dispatch(p->dtype, p->ndim, p->j6, FwdFn{p, s});
}

int ragged_interp_adj(tkbn_ragged_plan p, cudaStream_t s) {
  if (!p) return set_error(TKBN_ERR_INVALID, "ragged plan is null");
  return ragged_dispatch(p->dtype, p->ndim, p->j6, AdjFn{p, s});
}

}  // namespace tkbn_host

TKBN_DEFINE_STATUS_READER(status_interp)
