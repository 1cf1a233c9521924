// K1: trajectory layout — bin-sort of k-space points by grid tile.
//
// Replaces the float-key sort of the reference adjoint (sort_one_batch,
// torchkbnufft/_nufft/interp.py:551-584). Points are keyed by the tile that
// holds the first cell of their J^d footprint; a stable radix sort keeps the
// original point order inside each tile, so consecutive points of a spoke stay
// adjacent. The sorted coordinates, original indices and a list of work items
// (at most `chunk` points of one tile each) are written to a caller-owned
// workspace; the interpolation kernels read only that workspace.

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "tkbn_common.cuh"
#include "geo_host.cuh"

namespace tkbn {

template <typename R>
__global__ void k_point_keys(Geo<R> geo, const R* __restrict__ omega, int64_t M, int64_t ntraj,
                             uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t n = M * ntraj;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = i / M;
    const int64_t m = i - t * M;
    int key = 0;
    bool ok = true;
    for (int d = 0; d < geo.ndim; ++d) {
      R om = omega[(t * geo.ndim + d) * M + m];
      R tm;
      int base;
      ok = ok && base_index<R>(om, geo.gam[d], geo.halfJ[d], &tm, &base);
      int tile = pmod(base, geo.K[d]) / geo.T[d];
      key = key * geo.ntile[d] + tile;
    }
    if (!ok) {
      atomicOr(&g_status, kStatusNonFinite);
      key = 0;
    }
    keys[i] = (uint32_t)(t * geo.ntiles + key);
    vals[i] = (int32_t)i;
  }
}

__global__ void k_count_keys(const uint32_t* __restrict__ keys, int64_t n, int32_t* __restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&counts[keys[i]], 1);
}

__global__ void k_items_per_key(const int32_t* __restrict__ counts, int64_t nkeys, int chunk,
                                int32_t* __restrict__ nit) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nkeys; k += (int64_t)gridDim.x * blockDim.x)
    nit[k] = (counts[k] + chunk - 1) / chunk;
}

__global__ void k_fill_items(const int32_t* __restrict__ counts, const int32_t* __restrict__ tile_off,
                             const int32_t* __restrict__ nit, const int32_t* __restrict__ item_off, int64_t nkeys,
                             int chunk, Item* __restrict__ items, int64_t* __restrict__ hdr) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nkeys; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = counts[k];
    const int o = item_off[k];
    for (int q = 0; q < nit[k]; ++q) {
      Item it;
      it.key = (int)k;
      it.start = tile_off[k] + q * chunk;
      it.len = min(chunk, c - q * chunk);
      it.pad = 0;
      items[o + q] = it;
    }
    if (k == nkeys - 1) hdr[0] = (int64_t)o + nit[k];
  }
}

// Work items are ordered longest first, so that a grid-stride walk over them
// (CTA k takes items k, k + grid, ...) schedules the heavy k-space-centre tiles
// in the first wave (longest-processing-time-first). Items of at most `light`
// points share one key, so the stable sort keeps them in tile order after the
// heavy ones: CTAs that run at the same time then stage neighbouring tiles,
// whose halos overlap in L2 (3D layouts; light = 0 orders every item by length).
__global__ void k_item_keys(const Item* __restrict__ items, const int64_t* __restrict__ hdr, int64_t max_items,
                            int chunk, int light, uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t nitems = hdr[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < max_items; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = i < nitems ? (uint32_t)(chunk - max(items[i].len, light)) : (uint32_t)(chunk + 1);
    vals[i] = (int32_t)i;
  }
}

__global__ void k_gather_items(const Item* __restrict__ items, const int32_t* __restrict__ order, int64_t max_items,
                               Item* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < max_items; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = items[order[i]];
}

// Adjoint work of an output tile: the points of every tile whose footprints
// can reach it (itself and up to nsrc-1 tiles before it in each dim). The
// sort key is the bitwise complement, so an ascending sort puts the heaviest
// tile first.
template <typename R>
__global__ void k_tile_work(Geo<R> geo, const int32_t* __restrict__ counts, const int32_t* __restrict__ vcount,
                            int64_t nkeys, SrcSpan span, int W, int32_t* __restrict__ work,
                            int32_t* __restrict__ nsub) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nkeys; k += (int64_t)gridDim.x * blockDim.x) {
    int64_t w = 0;
    if (vcount) {
      w = vcount[k];
    } else {
      const int64_t t = k / geo.ntiles;
      int rem = (int)(k - t * geo.ntiles);
      int td[kMaxDim] = {0, 0, 0};
      for (int d = geo.ndim - 1; d >= 0; --d) {
        td[d] = rem % geo.ntile[d];
        rem /= geo.ntile[d];
      }
      for (int combo = 0; combo < span.ncombo; ++combo) w += counts[t * geo.ntiles + source_tile(geo, span, td, combo)];
    }
    work[k] = (int32_t)w;
    nsub[k] = w > W ? (int32_t)((w + W - 1) / W) : 1;
  }
}

// 2D owned tiles: one CTA per output tile walks the points of its source
// tiles (in source-tile order, then sorted order — the order the adjoint
// accumulates them in), 1024 candidates at a time, 4 consecutive ones per
// thread, and keeps those whose footprint reaches the tile, with the
// footprint's first row and column relative to the tile origin (negative
// when the footprint starts in an earlier tile; periodic). A block-wide
// exclusive scan of the per-thread counts keeps the order. The first pass
// (voff == nullptr) counts, the second writes at voff[key].
// In 3D the entry packs the row and column offsets: {i, m, rz, (ry & 0xffff) | (rx << 16)}.
constexpr int kValidThreads = 256;
template <typename R, int D>
__global__ void __launch_bounds__(kValidThreads) k_tile_valid(Geo<R> geo, const int32_t* __restrict__ counts,
                                                              const int32_t* __restrict__ tile_off,
                                                              const R* __restrict__ tm, const int32_t* __restrict__ vals,
                                                              int64_t n, int64_t M, int64_t nkeys, SrcSpan span,
                                                              const int32_t* __restrict__ voff,
                                                              int32_t* __restrict__ vcount, int4* __restrict__ vlist) {
  constexpr int MAXCOMBO = D == 2 ? 16 : 27;
  __shared__ int s_start[MAXCOMBO], s_pre[MAXCOMBO + 1], s_warp[kValidThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t key = blockIdx.x; key < nkeys; key += gridDim.x) {
    const int64_t t = key / geo.ntiles;
    int rem = (int)(key - t * geo.ntiles);
    int td[kMaxDim] = {0, 0, 0};
#pragma unroll
    for (int d = D - 1; d >= 0; --d) {
      td[d] = rem % geo.ntile[d];
      rem /= geo.ntile[d];
    }
    int origin[D], ext[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      origin[d] = td[d] * geo.T[d];
      ext[d] = min(geo.T[d], geo.K[d] - origin[d]);
    }
    __syncthreads();  // the previous key is done with the shared lists
    if ((int)threadIdx.x < span.ncombo) {
      const int64_t skey = t * geo.ntiles + source_tile(geo, span, td, threadIdx.x);
      s_start[threadIdx.x] = tile_off[skey];
      s_pre[threadIdx.x + 1] = counts[skey];
    }
    if (threadIdx.x == 0) s_pre[0] = 0;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int l = 0; l < span.ncombo; ++l) s_pre[l + 1] += s_pre[l];
    __syncthreads();
    const int total = s_pre[span.ncombo];
    const int64_t out0 = voff ? voff[key] : 0;
    int cnt = 0;
    for (int q0 = 0; q0 < total; q0 += 4 * kValidThreads) {
      bool valid[4];
      int idx[4], ry[4], rx[4];
      int mine = 0, l = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int q = q0 + 4 * (int)threadIdx.x + k;
        valid[k] = false;
        idx[k] = ry[k] = rx[k] = 0;
        if (q < total) {
          while (s_pre[l + 1] <= q) ++l;
          const int i = s_start[l] + (q - s_pre[l]);
          bool v = true;
          int r[D];
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const R f = floor(sub_rn(tm[d * n + i], geo.halfJ[d]));
            const bool fin = fabs(f) < R(1 << 30);
            const int w = fin ? wrap_cell(1 + (int)f, geo.K[d]) : 0;
            int rr = w - origin[d];
            if (rr >= geo.T[d]) rr -= geo.K[d];
            v = v && fin && (rr > -geo.J[d]) && (rr < ext[d]);
            r[d] = rr;
          }
          valid[k] = v;
          idx[k] = i;
          ry[k] = r[0];
          rx[k] = D == 2 ? r[1] : ((r[1 % D] & 0xffff) | (r[2 % D] << 16));
          mine += v ? 1 : 0;
        }
      }
      // block-wide exclusive scan of the per-thread counts
      int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) s_warp[warp] = incl;
      __syncthreads();
      int before = 0, chunk = 0;
#pragma unroll
      for (int w = 0; w < kValidThreads / 32; ++w) {
        const int c = s_warp[w];
        before += w < warp ? c : 0;
        chunk += c;
      }
      if (voff) {
        int pos = cnt + before + incl - mine;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (valid[k]) vlist[out0 + pos++] = make_int4(idx[k], (int)(vals[idx[k]] - t * M), ry[k], rx[k]);
      }
      cnt += chunk;
      __syncthreads();  // s_warp is rewritten by the next chunk
    }
    if (!voff && threadIdx.x == 0) vcount[key] = cnt;
  }
}

// Lists sorted by footprint start in the last two dims, stable (equal starts
// keep list order), one warp per tile: count the starts
// (k = (rx + ox) * ny + ry + oy; rx, ry the column and row offsets, packed in
// the entry's last word in 3D), scan the counts into a koff row and place the
// entries 32 at a time in list order, ranking equal starts within the 32 by
// lane. chunk == 0: the whole list, koff row = tile. chunk > 0: each chunk of
// `chunk` entries separately, koff row (voff[tile] + first) / chunk + tile,
// and the output entry carries its position in the chunk in place of m.
constexpr int kSortWarps = 8, kSortMaxKeys = 1024;
__global__ void __launch_bounds__(kSortWarps * 32)
    k_tile_keysort(int64_t nkeys, int d3, int chunk, int ny, int oy, int ox, int nk, const int32_t* __restrict__ voff,
                   const int32_t* __restrict__ vcount, const int4* __restrict__ vin, int4* __restrict__ vout,
                   int32_t* __restrict__ koff) {
  extern __shared__ int32_t s_cur[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t* cur = s_cur + warp * (nk + 1);
  auto skey = [&](const int4& e) {
    const int ry = d3 ? (int)(short)(e.w & 0xffff) : e.z, rx = d3 ? (e.w >> 16) : e.w;
    return (rx + ox) * ny + ry + oy;
  };
  for (int64_t key = (int64_t)blockIdx.x * kSortWarps + warp; key < nkeys; key += (int64_t)gridDim.x * kSortWarps) {
    const int64_t tbase = voff[key];
    const int tcnt = vcount[key];
    const int span = chunk > 0 ? chunk : (tcnt > 0 ? tcnt : 1);
    for (int first = 0; first < tcnt || (first == 0 && chunk == 0); first += span) {
      const int64_t base = tbase + first;
      const int cnt = min(span, tcnt - first);
      for (int k = lane; k <= nk; k += 32) cur[k] = 0;
      __syncwarp();
      for (int q = lane; q < cnt; q += 32) atomicAdd(&cur[skey(vin[base + q])], 1);
      __syncwarp();
      // exclusive scan of cur[0 .. nk]: lane l takes a run of `per` entries
      const int per = (nk + 1 + 31) / 32, lo = lane * per, hi = min(lo + per, nk + 1);
      int sum = 0;
      for (int k = lo; k < hi; ++k) sum += cur[k];
      int incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      int run = incl - sum;
      for (int k = lo; k < hi; ++k) {
        const int c = cur[k];
        cur[k] = run;
        run += c;
      }
      __syncwarp();
      const int64_t row = chunk > 0 ? base / chunk + key : key;
      int32_t* ko = koff + row * (nk + 1);
      for (int k = lane; k <= nk; k += 32) ko[k] = cur[k];
      __syncwarp();
      for (int q0 = 0; q0 < cnt; q0 += 32) {
        const int q = q0 + lane;
        const bool act = q < cnt;
        int4 e = make_int4(0, 0, 0, 0);
        int k = nk;  // idle lanes share the end slot and write nothing
        if (act) {
          e = vin[base + q];
          k = skey(e);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, k);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        const int pos = cur[k] + rank;
        __syncwarp();
        if (act && rank == 0) cur[k] += __popc(peers);
        __syncwarp();
        if (chunk > 0) e.y = q;
        if (act) vout[base + pos] = e;
      }
      __syncwarp();
      if (chunk == 0) break;
    }
  }
}

// Adjoint sub-jobs: candidates [start, start+len) of output tile `key`; pad = 1
// when the tile is split over several sub-jobs (their results are added with
// atomics into a pre-zeroed tile; unsplit tiles are written with plain stores).
__global__ void k_fill_subjobs(const int32_t* __restrict__ work, const int32_t* __restrict__ nsub,
                               const int32_t* __restrict__ suboff, int64_t nkeys, int W, Item* __restrict__ jobs,
                               int64_t* __restrict__ hdr) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nkeys; k += (int64_t)gridDim.x * blockDim.x) {
    const int ns = nsub[k];
    for (int q = 0; q < ns; ++q) {
      Item it;
      it.key = (int)k;
      it.start = q * W;
      it.len = min(W, work[k] - q * W);
      it.pad = ns > 1 ? 1 : 0;
      jobs[suboff[k] + q] = it;
    }
    if (k == nkeys - 1) hdr[1] = (int64_t)suboff[k] + ns;
  }
}

__global__ void k_subjob_keys(const Item* __restrict__ jobs, const int64_t* __restrict__ hdr, int64_t max_jobs, int W,
                              uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t n = hdr[1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < max_jobs; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = i < n ? (uint32_t)(W - jobs[i].len) : (uint32_t)(W + 1);
    vals[i] = (int32_t)i;
  }
}

// Per sorted point: normalised frequency tm_d = omega_d / gam_d and the
// fftshift phase exp(i sum_d omega_d n_shift_d), both with the reference's
// rounding (see base_index / phase_arg). The interpolation kernels read only
// these, never omega.
template <typename R>
__global__ void k_sorted_points(Geo<R> geo, const R* __restrict__ omega, const int32_t* __restrict__ vals, int64_t M,
                                int64_t n, R* __restrict__ tm, cplx<R>* __restrict__ ph) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = vals[i];
    const int64_t t = v / M;
    const int64_t m = v - t * M;
    R om[kMaxDim];
    for (int d = 0; d < geo.ndim; ++d) {
      om[d] = omega[(t * geo.ndim + d) * M + m];
      tm[d * n + i] = div_rn(om[d], geo.gam[d]);
    }
    R a = mul_rn(om[0], geo.nshift[0]);
    for (int d = 1; d < geo.ndim; ++d) a = add_rn(a, mul_rn(om[d], geo.nshift[d]));
    R sn, cs;
    sincos_acc(a, &sn, &cs);
    ph[i] = mk<R>(cs, sn);
  }
}

}  // namespace tkbn

namespace tkbn_host {

static thread_local char g_errbuf[512];
const char* last_error() { return g_errbuf; }

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof(g_errbuf), fmt, ap);
  va_end(ap);
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TKBN_OK;
  return set_error(TKBN_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int resident_grid(const void* kernel, int threads, size_t smem, int64_t* blocks) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, int, size_t>, int64_t> cache;
  // the kernel's shared-memory limit only ever grows (a launch may use any
  // size up to it), so a cached launch shape stays valid
  static std::map<std::pair<int, const void*>, size_t> limit;
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  const auto key = std::make_tuple(dev, kernel, threads, smem);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *blocks = it->second;
    return TKBN_OK;
  }
  size_t& lim = limit[std::make_pair(dev, kernel)];
  if (smem > lim) {
    if ((rc = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "smem attribute")))
      return rc;
    lim = smem;
  }
  int sms = 0, per_sm = 0;
  if ((rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))) return rc;
  if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem), "occupancy")))
    return rc;
  if (per_sm < 1) return set_error(TKBN_ERR_UNSUPPORTED, "kernel cannot be resident with %zu B of shared memory", smem);
  *blocks = (int64_t)per_sm * sms;
  cache[key] = *blocks;
  return TKBN_OK;
}

void default_tiles(const tkbn_geometry* g, int tile[3], int* chunk) {
  for (int d = 0; d < 3; ++d) tile[d] = 1;
  if (g->ndim == 1) {
    tile[0] = 128;
  } else if (g->ndim == 2) {
    // 16 rows x 14 columns: a 21 x 19 forward patch of 16 complex64 coil
    // planes is 51 KB, so four 256-thread CTAs fit an SM; the register
    // adjoint's 16-coil jobs give each of the 8 warps two of the 16 rows.
    tile[0] = 16;
    tile[1] = 14;
  } else {
    // 4 x 8 x 8: 32 (z, y) rows of 8 cells for the register adjoint
    tile[0] = 4;
    tile[1] = tile[2] = 8;
  }
  *chunk = 1024;
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

int points_layout(const tkbn_geometry* g, const tkbn_points_desc* p, PointsLayout* L) {
  if (!g || !p || !L) return set_error(TKBN_ERR_INVALID, "null argument");
  if (g->ndim < 1 || g->ndim > 3) return set_error(TKBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3 (got %d)", g->ndim);
  if (p->npts < 0 || p->ntraj < 1) return set_error(TKBN_ERR_INVALID, "npts must be >= 0 and ntraj >= 1");
  int dtile[3], dchunk;
  default_tiles(g, dtile, &dchunk);
  int64_t ntiles = 1;
  for (int d = 0; d < g->ndim; ++d) {
    if (g->grid_size[d] < 1 || g->grid_size[d] > (1 << 24))
      return set_error(TKBN_ERR_INVALID, "grid_size[%d] out of range", d);
    int t = p->tile[d] > 0 ? p->tile[d] : dtile[d];
    if (t > g->grid_size[d]) t = (int)g->grid_size[d];
    L->tile[d] = t;
    L->ntile[d] = (int)((g->grid_size[d] + t - 1) / t);
    ntiles *= L->ntile[d];
  }
  for (int d = g->ndim; d < 3; ++d) {
    L->tile[d] = 1;
    L->ntile[d] = 1;
  }
  L->chunk = p->chunk > 0 ? p->chunk : dchunk;
  L->nkeys = ntiles * p->ntraj;
  L->npts_total = p->npts * p->ntraj;
  if (L->nkeys >= (int64_t)1 << 31 || L->npts_total >= (int64_t)1 << 31)
    return set_error(TKBN_ERR_INVALID, "trajectory too large for 32-bit point indices");
  L->max_items = L->nkeys + (L->npts_total + L->chunk - 1) / L->chunk;
  int bits = 1;
  while (((int64_t)1 << bits) < L->nkeys) ++bits;
  L->key_bits = bits;

  const int64_t n = L->npts_total > 0 ? L->npts_total : 1;
  const size_t rsize = g->dtype == TKBN_C64 ? 4 : 8;
  int ibits = 1;
  while (((int64_t)1 << ibits) <= L->chunk + 1) ++ibits;
  L->item_key_bits = ibits;
  size_t cub_sort = 0, cub_scan = 0, cub_isort = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, cub_sort, (uint32_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)n, 0, bits);
  cub::DeviceScan::ExclusiveSum(nullptr, cub_scan, (int32_t*)nullptr, (int32_t*)nullptr, (int)L->nkeys);
  cub::DeviceRadixSort::SortPairs(nullptr, cub_isort, (uint32_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)L->max_items, 0, ibits);
  L->cub_bytes = cub_sort > cub_scan ? cub_sort : cub_scan;
  if (cub_isort > L->cub_bytes) L->cub_bytes = cub_isort;
  size_t cub_tsort = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, cub_tsort, (uint32_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)L->nkeys, 0, 32);
  if (cub_tsort > L->cub_bytes) L->cub_bytes = cub_tsort;
  // output-tile sources for the adjoint
  L->span.ncombo = 1;
  L->owned_ok = true;
  for (int d = 0; d < 3; ++d) {
    if (d >= g->ndim) {
      L->span.nsrc[d] = 1;
      continue;
    }
    const int T = L->tile[d];
    const int lastw = (int)(g->grid_size[d] - (int64_t)(L->ntile[d] - 1) * T);
    const int minw = lastw < T ? lastw : T;
    int ns = 1 + (g->numpoints[d] - 1 + minw - 1) / minw;
    if (ns > L->ntile[d]) ns = L->ntile[d];
    L->span.nsrc[d] = ns;
    L->span.ncombo *= ns;
    if (g->grid_size[d] < (int64_t)T + g->numpoints[d] - 1) L->owned_ok = false;
  }
  // adjoint sub-jobs: at most adj_chunk candidates (list entries in 2D) each
  L->adj_chunk = (g->flags & TKBN_ADJ_DETERMINISTIC) ? (1 << 30) : 1024;
  // the owned-tile kernels' source limits: 16 source tiles in 2D, 27 in 3D
  L->vlist = L->owned_ok && !(g->flags & TKBN_LAYOUT_FORWARD_ONLY) &&
             ((g->ndim == 2 && L->span.ncombo <= 16) || (g->ndim == 3 && L->span.ncombo <= 27));
  L->max_valid = L->vlist ? L->span.ncombo * L->npts_total : 0;
  // sort key of a list entry: (column offset, row offset) of the last two dims
  if (g->ndim >= 2) {
    const int dr = g->ndim - 2, dc = g->ndim - 1;
    L->kny = L->tile[dr] + g->numpoints[dr] - 1;
    L->knk = L->kny * (L->tile[dc] + g->numpoints[dc] - 1);
  } else {
    L->kny = L->knk = 0;
  }
  // chunk-sorted copies for the register adjoints: 2D 16 x 14 and 3D 4 x 8 x 8
  // tiles, complex64, J = 6
  bool j6 = true;
  for (int d = 0; d < g->ndim; ++d) j6 = j6 && g->numpoints[d] == 6;
  const bool regtile = (g->ndim == 2 && L->tile[0] == 16 && L->tile[1] == 14) ||
                       (g->ndim == 3 && L->tile[0] == 4 && L->tile[1] == 8 && L->tile[2] == 8);
  L->ksort = false;
  L->csort = L->vlist && g->dtype == TKBN_C64 && j6 && regtile && L->adj_chunk % tkbn::kListChunk == 0 &&
             L->knk <= tkbn::kSortMaxKeys;
  L->pfac = L->csort && g->ndim == 2;
  L->lfix = L->csort && g->ndim == 3;
  L->pfac3 = L->lfix;
  L->koff_rows = L->ksort ? L->nkeys : (L->csort ? L->max_valid / tkbn::kListChunk + L->nkeys + 1 : 0);
  L->max_subjobs = 2 * L->nkeys + (L->span.ncombo * L->npts_total + L->adj_chunk - 1) / L->adj_chunk;
  int sbits = 1;
  while (((int64_t)1 << sbits) <= L->adj_chunk + 1) ++sbits;
  L->sj_key_bits = sbits;
  size_t cub_ssort = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, cub_ssort, (uint32_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)L->max_subjobs, 0, sbits);
  if (cub_ssort > L->cub_bytes) L->cub_bytes = cub_ssort;

  size_t o = 0;
  L->off_hdr = o;
  o = align_up(o + 64);
  L->off_keys_in = o;
  o = align_up(o + 4 * n);
  L->off_vals_in = o;
  o = align_up(o + 4 * n);
  L->off_keys = o;
  o = align_up(o + 4 * n);
  L->off_vals = o;
  o = align_up(o + 4 * n);
  L->off_counts = o;
  o = align_up(o + 4 * L->nkeys);
  L->off_tile_off = o;
  o = align_up(o + 4 * (L->nkeys + 1));
  L->off_nit = o;
  o = align_up(o + 4 * L->nkeys);
  L->off_item_off = o;
  o = align_up(o + 4 * (L->nkeys + 1));
  L->off_items = o;
  o = align_up(o + sizeof(tkbn::Item) * L->max_items);
  L->off_items_raw = o;
  o = align_up(o + sizeof(tkbn::Item) * L->max_items);
  L->off_ikeys_in = o;
  o = align_up(o + 4 * L->max_items);
  L->off_ikeys = o;
  o = align_up(o + 4 * L->max_items);
  L->off_ivals_in = o;
  o = align_up(o + 4 * L->max_items);
  L->off_ivals = o;
  o = align_up(o + 4 * L->max_items);
  L->off_tile_work = o;
  o = align_up(o + 4 * L->nkeys);
  L->off_tile_nsub = o;
  o = align_up(o + 4 * L->nkeys);
  L->off_tile_suboff = o;
  o = align_up(o + 4 * (L->nkeys + 1));
  L->off_sj_raw = o;
  o = align_up(o + sizeof(tkbn::Item) * L->max_subjobs);
  L->off_adj_jobs = o;
  o = align_up(o + sizeof(tkbn::Item) * L->max_subjobs);
  L->off_sj_keys_in = o;
  o = align_up(o + 4 * L->max_subjobs);
  L->off_sj_keys = o;
  o = align_up(o + 4 * L->max_subjobs);
  L->off_sj_vals_in = o;
  o = align_up(o + 4 * L->max_subjobs);
  L->off_sj_vals = o;
  o = align_up(o + 4 * L->max_subjobs);
  L->off_vcount = o;
  o = align_up(o + (L->vlist ? 4 * L->nkeys : 0));
  L->off_voff = o;
  o = align_up(o + (L->vlist ? 4 * (L->nkeys + 1) : 0));
  L->off_vlist = o;
  o = align_up(o + sizeof(int4) * L->max_valid);
  L->off_vtmp = o;
  o = align_up(o + (L->ksort ? sizeof(int4) * L->max_valid : 0));
  L->off_vsort = o;
  o = align_up(o + (L->csort ? sizeof(int4) * L->max_valid : 0));
  L->off_koff = o;
  o = align_up(o + 4 * (size_t)L->koff_rows * (L->knk + 1));
  L->off_pfac = o;
  o = align_up(o + (L->pfac ? (size_t)L->npts_total * 12 * 8 + 512 : 0));  // + linear-phase tables
  L->off_lfix = o;
  o = align_up(o + (L->lfix ? (size_t)4 * L->npts_total + 64 : 0));
  L->off_pfac3 = o;
  o = align_up(o + (L->pfac3 ? (size_t)tkbn::kLp3PRec * sizeof(float) * L->npts_total : 0));
  L->off_coords = o;
  o = align_up(o + rsize * g->ndim * n);
  L->off_phase = o;
  o = align_up(o + 2 * rsize * n);
  L->off_cub = o;
  o = align_up(o + L->cub_bytes);
  L->total = o;
  return TKBN_OK;
}

template <typename R>
static int build_impl(const tkbn_geometry* g, const tkbn_points_desc* p, const PointsLayout& L, const void* omega,
                      char* ws, cudaStream_t s) {
  using namespace tkbn;
  Geo<R> geo = make_geo<R>(g, &L, nullptr, nullptr);
  const int64_t n = L.npts_total;
  uint32_t* keys_in = (uint32_t*)(ws + L.off_keys_in);
  int32_t* vals_in = (int32_t*)(ws + L.off_vals_in);
  uint32_t* keys = (uint32_t*)(ws + L.off_keys);
  int32_t* vals = (int32_t*)(ws + L.off_vals);
  int32_t* counts = (int32_t*)(ws + L.off_counts);
  int32_t* tile_off = (int32_t*)(ws + L.off_tile_off);
  int32_t* nit = (int32_t*)(ws + L.off_nit);
  int32_t* item_off = (int32_t*)(ws + L.off_item_off);
  Item* items = (Item*)(ws + L.off_items);
  Item* items_raw = (Item*)(ws + L.off_items_raw);
  uint32_t* ikeys_in = (uint32_t*)(ws + L.off_ikeys_in);
  uint32_t* ikeys = (uint32_t*)(ws + L.off_ikeys);
  int32_t* ivals_in = (int32_t*)(ws + L.off_ivals_in);
  int32_t* ivals = (int32_t*)(ws + L.off_ivals);
  R* coords = (R*)(ws + L.off_coords);
  int64_t* hdr = (int64_t*)(ws + L.off_hdr);
  void* cubtmp = ws + L.off_cub;

  int rc;
  if ((rc = check_cuda(cudaMemsetAsync(ws + L.off_hdr, 0, 64, s), "memset header"))) return rc;
  if ((rc = check_cuda(cudaMemsetAsync(counts, 0, 4 * L.nkeys, s), "memset counts"))) return rc;
  const int threads = 256;
  auto blocks_for = [&](int64_t work) {
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
  };
  if (n > 0) {
    k_point_keys<R><<<blocks_for(n), threads, 0, s>>>(geo, (const R*)omega, p->npts, p->ntraj, keys_in, vals_in);
    size_t tb = L.cub_bytes;
    if (cub::DeviceRadixSort::SortPairs(cubtmp, tb, keys_in, keys, vals_in, vals, (int)n, 0, L.key_bits, s) !=
        cudaSuccess)
      return set_error(TKBN_ERR_CUDA, "radix sort failed");
    k_count_keys<<<blocks_for(n), threads, 0, s>>>(keys, n, counts);
  }
  k_items_per_key<<<blocks_for(L.nkeys), threads, 0, s>>>(counts, L.nkeys, L.chunk, nit);
  size_t tb = L.cub_bytes;
  if (cub::DeviceScan::ExclusiveSum(cubtmp, tb, counts, tile_off, (int)L.nkeys, s) != cudaSuccess)
    return set_error(TKBN_ERR_CUDA, "scan failed");
  tb = L.cub_bytes;
  if (cub::DeviceScan::ExclusiveSum(cubtmp, tb, nit, item_off, (int)L.nkeys, s) != cudaSuccess)
    return set_error(TKBN_ERR_CUDA, "scan failed");
  k_fill_items<<<blocks_for(L.nkeys), threads, 0, s>>>(counts, tile_off, nit, item_off, L.nkeys, L.chunk, items_raw,
                                                       hdr);
  // 3D: items of up to 256 points stay in tile order (their 9 x 13 x 13 patch halos are reread from L2)
  const int light = g->ndim == 3 ? (L.chunk < 256 ? L.chunk : 256) : 0;
  k_item_keys<<<blocks_for(L.max_items), threads, 0, s>>>(items_raw, hdr, L.max_items, L.chunk, light, ikeys_in,
                                                          ivals_in);
  tb = L.cub_bytes;
  if (cub::DeviceRadixSort::SortPairs(cubtmp, tb, ikeys_in, ikeys, ivals_in, ivals, (int)L.max_items, 0,
                                      L.item_key_bits, s) != cudaSuccess)
    return set_error(TKBN_ERR_CUDA, "item sort failed");
  k_gather_items<<<blocks_for(L.max_items), threads, 0, s>>>(items_raw, ivals, L.max_items, items);
  if (n > 0)
    k_sorted_points<R><<<blocks_for(n), threads, 0, s>>>(geo, (const R*)omega, vals, p->npts, n, coords,
                                                         (cplx<R>*)(ws + L.off_phase));
  // 2D: per output tile, the points that reach it
  int32_t* vcount = nullptr;
  if (L.vlist) {
    vcount = (int32_t*)(ws + L.off_vcount);
    int32_t* voff = (int32_t*)(ws + L.off_voff);
    int4* vlist = (int4*)(ws + L.off_vlist);
    const int wblocks = (int)(L.nkeys < 152 * 8 ? L.nkeys : 152 * 8);
    auto kv = g->ndim == 2 ? k_tile_valid<R, 2> : k_tile_valid<R, 3>;
    kv<<<wblocks, kValidThreads, 0, s>>>(geo, counts, tile_off, coords, vals, n, p->npts, L.nkeys, L.span, nullptr,
                                         vcount, vlist);
    tb = L.cub_bytes;
    if (cub::DeviceScan::ExclusiveSum(cubtmp, tb, vcount, voff, (int)L.nkeys, s) != cudaSuccess)
      return set_error(TKBN_ERR_CUDA, "scan failed");
    int4* vdst = L.ksort ? (int4*)(ws + L.off_vtmp) : vlist;  // 3D: sorted into vlist below
    kv<<<wblocks, kValidThreads, 0, s>>>(geo, counts, tile_off, coords, vals, n, p->npts, L.nkeys, L.span, voff,
                                         vcount, vdst);
    if (L.ksort || L.csort) {
      const int64_t sb = (L.nkeys + kSortWarps - 1) / kSortWarps;
      const size_t ssmem = (size_t)kSortWarps * (L.knk + 1) * sizeof(int32_t);
      k_tile_keysort<<<(int)(sb < 152 * 8 ? sb : 152 * 8), kSortWarps * 32, ssmem, s>>>(
          L.nkeys, g->ndim == 3, L.csort ? kListChunk : 0, L.kny, g->numpoints[g->ndim - 2] - 1,
          g->numpoints[g->ndim - 1] - 1, L.knk, voff, vcount, vdst, L.csort ? (int4*)(ws + L.off_vsort) : vlist,
          (int32_t*)(ws + L.off_koff));
    }
  }
  // adjoint sub-jobs (output tiles, heavy ones split), longest first
  {
    int32_t* work = (int32_t*)(ws + L.off_tile_work);
    int32_t* nsub = (int32_t*)(ws + L.off_tile_nsub);
    int32_t* suboff = (int32_t*)(ws + L.off_tile_suboff);
    Item* sj_raw = (Item*)(ws + L.off_sj_raw);
    uint32_t* sk_in = (uint32_t*)(ws + L.off_sj_keys_in);
    uint32_t* sk = (uint32_t*)(ws + L.off_sj_keys);
    int32_t* sv_in = (int32_t*)(ws + L.off_sj_vals_in);
    int32_t* sv = (int32_t*)(ws + L.off_sj_vals);
    k_tile_work<R><<<blocks_for(L.nkeys), threads, 0, s>>>(geo, counts, vcount, L.nkeys, L.span, L.adj_chunk, work,
                                                           nsub);
    tb = L.cub_bytes;
    if (cub::DeviceScan::ExclusiveSum(cubtmp, tb, nsub, suboff, (int)L.nkeys, s) != cudaSuccess)
      return set_error(TKBN_ERR_CUDA, "scan failed");
    k_fill_subjobs<<<blocks_for(L.nkeys), threads, 0, s>>>(work, nsub, suboff, L.nkeys, L.adj_chunk, sj_raw, hdr);
    k_subjob_keys<<<blocks_for(L.max_subjobs), threads, 0, s>>>(sj_raw, hdr, L.max_subjobs, L.adj_chunk, sk_in,
                                                                 sv_in);
    tb = L.cub_bytes;
    if (cub::DeviceRadixSort::SortPairs(cubtmp, tb, sk_in, sk, sv_in, sv, (int)L.max_subjobs, 0, L.sj_key_bits, s) !=
        cudaSuccess)
      return set_error(TKBN_ERR_CUDA, "sub-job sort failed");
    k_gather_items<<<blocks_for(L.max_subjobs), threads, 0, s>>>(sj_raw, sv, L.max_subjobs,
                                                                  (Item*)(ws + L.off_adj_jobs));
  }
  return check_cuda(cudaGetLastError(), "points build launch");
}

int points_build(const tkbn_geometry* g, const tkbn_points_desc* p, const void* omega, void* ws, size_t bytes,
                 cudaStream_t s) {
  PointsLayout L;
  int rc = points_layout(g, p, &L);
  if (rc) return rc;
  if (!ws) return set_error(TKBN_ERR_INVALID, "workspace is null");
  if (bytes < L.total) return set_error(TKBN_ERR_INVALID, "workspace too small: %zu < %zu", bytes, L.total);
  if (p->npts > 0 && !omega) return set_error(TKBN_ERR_INVALID, "omega is null");
  if (g->dtype == TKBN_C64) return build_impl<float>(g, p, L, omega, (char*)ws, s);
  if (g->dtype == TKBN_C128) return build_impl<double>(g, p, L, omega, (char*)ws, s);
  return set_error(TKBN_ERR_UNSUPPORTED, "unsupported dtype %d", g->dtype);
}

}  // namespace tkbn_host

TKBN_DEFINE_STATUS_READER(status_points)
