// K4 with coil-part lanes: the 2D complex64 adjoint interpolation for
// linear-phase tables (table_interp_adjoint, torchkbnufft/_nufft/interp.py:
// 587-726), on 16 x 4 output tiles.
//
// A warp owns one output tile of one batch item and up to 16 coils. Lane
// (group g, coil c, part p) keeps part p (real or imaginary) of the tile's 64
// cells for coil c in registers. With linear-phase tables every tap weight is
// real once the k-space value carries the entry's phase Q (see kLpE0 in
// interp.cu), so the two parts accumulate independently: one FMA per tap and
// lane, and every lane of the warp updates the same cells. Register indices
// must be compile-time constants, so each 32-entry group of the tile's list
// is processed in runs of equal footprint start row ry (entries sorted by ry
// within the group, ranks precomputed by the layout build): the run's code
// knows ry, and the entry's column start rx enters through four column
// factors MX[x] = mx[x - rx] (zero outside the footprint). With fewer than
// 16 coils per job the 16 / CC lane groups take the run's entries in turn and
// their tiles are summed by shuffles before the write-out.
//
// Each entry's record {MX[4], my[6], Q} (Q = P Ey[2 + ry] Ex[2 + rx], the
// entry's linear-phase factor) is computed once per layout and table set by
// k_atile_records, with the per-point factor pre-pass, and stored in
// sorted-slot order. Staging is per warp and double-buffered: while a group
// is processed, the next group's records and k-space values are in flight
// (cp.async, k-space values copied in list order, which keeps a radial
// spoke's consecutive samples together). No CTA barrier is involved. A group
// is walked key by key in a fixed order (static code per key, no indirect
// jumps), so the instruction stream stays sequential.
//
// The tile is multiplied by the per-cell phase R(y, x) and written once with
// 16-byte stores (two cells per lane after an exchange with the other part's
// lane); tiles split over several sub-jobs are accumulated with atomics into
// tiles zeroed first. Points the linear-phase form leaves out (factor record
// with P = 0) are added afterwards by k_adj_lp_fix (interp.cu).

#include <cstring>
#include <type_traits>

#include "geo_host.cuh"
#include "tkbn_common.cuh"

namespace tkbn {

constexpr int kCpWarps = 4;            // warps per CTA, each with its own jobs
constexpr int kCpSVS = kCpGroup + 1;   // coil stride (float2) of the staged k-space values: spreads banks
constexpr int kCpKeys = kCpTY + 5;     // footprint start rows ry = -5 .. 15
// linear-phase E tables, as written by the factor pre-pass (interp.cu):
// Ey[n] for n = -3 .. 17, then Ex[n] for n = -3 .. 15
constexpr int kCpE0 = 3, kCpEy = 21, kCpEx = 19;
constexpr int kCpEtabBytes = 512;      // E tables at the start of shared memory

// One staging buffer of a warp. rec[k][slot], k = 0..3: the entry record
// {MX0..3}, {my0..3}, {my4, my5, 0, 0}, {Q.x, -Q.y, Q.y, Q.x}; slots are the
// entries' ranks in the group sorted by footprint start row; k-major, so the
// lanes' 16-byte copies of one k are consecutive (no bank conflicts).
struct CpBuf {
  float4 rec[4][kCpGroup];
  int meta[kCpGroup];          // start-row key ry + 5 of each slot; 31 for an empty slot
  float2 sv[16 * kCpSVS];      // k-space values [coil][slot]
};

struct CpLaunch {
  const Item* jobs;      // sub-jobs {output tile key, first entry, entries, split}, longest first
  const int64_t* hdr;    // hdr[2] = number of sub-jobs
  const int4* vlist;     // per-tile lists {factor index, m, (ry + 5) | (rx + 5) << 8 | rank << 16, slot key}
  const int32_t* voff;   // first entry of each output tile
  const float4* arec;    // per list entry (sorted-slot order within its group): 4 float4 record
  const float2* etab;    // {Ey[kCpEy], Ex[kCpEx]}
  int64_t M, ntraj, B, C;
  int ncc;
  int64_t nbpt, gtot;
  int an1, per_t;        // output tiles per grid row, per trajectory
};

__device__ __forceinline__ void cp_async_16b(void* smem_dst, const void* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_8b(void* smem_dst, const void* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issues the copies of one group of a sub-job (list entries g0 .. g0 + nq)
// into buf; e is this lane's list entry of that group (valid when lane < nq).
template <int CC>
__device__ __forceinline__ void cp_stage(const CpLaunch& a, const float2* __restrict__ kdata, const int4& e,
                                         int64_t g0, int nq, int lane, int64_t b, int c0, int ncl, CpBuf& buf) {
  if (lane < nq) {
    const int rank = e.z >> 16;
    const float4* src = a.arec + (g0 + lane) * 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) cp_async_16b(&buf.rec[k][lane], src + k);
    buf.meta[lane] = e.w;
    const float2* vsrc = kdata + (b * a.C + c0) * a.M + e.y;
    float2* vdst = buf.sv + rank;
    if (ncl == CC) {
#pragma unroll
      for (int cl = 0; cl < CC; ++cl) {
        cp_async_8b(vdst + cl * kCpSVS, vsrc);
        vsrc += a.M;
      }
    } else {
#pragma unroll
      for (int cl = 0; cl < CC; ++cl) {
        if (cl < ncl)
          cp_async_8b(vdst + cl * kCpSVS, vsrc);
        else
          vdst[cl * kCpSVS] = make_float2(0.f, 0.f);
        vsrc += a.M;
      }
    }
  } else {
    buf.meta[lane] = 31;
  }
  cp_commit();
}

// Entry records of the staged group, per lane: r points at rec[0][slot] (the
// slot's other float4 sit kCpGroup and 2 kCpGroup float4 further, the lane's
// part of Q at q), v at the lane's coil's value of the slot.
struct CpPtr {
  const float4* r;
  const float2* q;
  const float2* v;
};

// N entries (slot stride `stride`) with footprint start row RY: part p of the
// k-space value times Q, then for every footprint row inside the tile
// acc[RY + j][x] += v my[j] MX[x]. Two entries are processed together so that
// their loads and products overlap.
template <int RY, int N>
__device__ __forceinline__ void cp_entries(const CpPtr& e, int stride, float (&acc)[kCpTY][kCpTX]) {
  float4 MX[N], m03[N], m45[N];
  float vp[N];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    const int o = n * stride;
    MX[n] = e.r[o];
    m03[n] = e.r[kCpGroup + o];
    m45[n] = e.r[2 * kCpGroup + o];
    const float2 qf = e.q[2 * o];
    const float2 v = e.v[o];
    vp[n] = fmaf(v.x, qf.x, v.y * qf.y);
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    if (RY + j >= 0 && RY + j < kCpTY) {
#pragma unroll
      for (int n = 0; n < N; ++n) {
        const float my = j < 4 ? (j == 0 ? m03[n].x : j == 1 ? m03[n].y : j == 2 ? m03[n].z : m03[n].w)
                               : (j == 4 ? m45[n].x : m45[n].y);
        const float w = vp[n] * my;
        acc[RY + j][0] = fmaf(w, MX[n].x, acc[RY + j][0]);
        acc[RY + j][1] = fmaf(w, MX[n].y, acc[RY + j][1]);
        acc[RY + j][2] = fmaf(w, MX[n].z, acc[RY + j][2]);
        acc[RY + j][3] = fmaf(w, MX[n].w, acc[RY + j][3]);
      }
    }
  }
}

// The runs of one staged group, key by key in a fixed order (keys absent
// from the group cost a bit test): a key's run is slots [lo, lo + count)
// (the slots are sorted by key); lane group grp takes slots lo + grp,
// lo + grp + G, ...
template <int CC, int K>
__device__ __forceinline__ void cp_keys(const CpPtr& base, unsigned present, int myk, int lo, int grp,
                                        float (&acc)[kCpTY][kCpTX]) {
  constexpr int G = 16 / CC;
  int next = lo;
  if (present & (1u << K)) {
    const int cnt = __popc(__ballot_sync(0xffffffffu, myk == K));
    next = lo + cnt;
    int p = lo + grp;
    CpPtr e{base.r + p, base.q + 2 * p, base.v + p};
#pragma unroll 1
    for (; p + G < next; p += 2 * G) {
      cp_entries<K - 5, 2>(e, G, acc);
      e.r += 2 * G;
      e.q += 4 * G;
      e.v += 2 * G;
    }
    if (p < next) cp_entries<K - 5, 1>(e, G, acc);
  }
  if constexpr (K + 1 < kCpKeys) cp_keys<CC, K + 1>(base, present, myk, next, grp, acc);
}

template <int CC>
__global__ void __launch_bounds__(kCpWarps * 32, 4)
    k_adj_cp(Geo<float> geo, CpLaunch a, const float2* __restrict__ kdata, float2* __restrict__ grid) {
  static_assert(CC >= 1 && CC <= 16 && (CC & (CC - 1)) == 0, "coils per job");
  constexpr int G = 16 / CC;
  extern __shared__ __align__(16) unsigned char smem[];
  float2* sE = reinterpret_cast<float2*>(smem);
  for (int t = threadIdx.x; t < kCpEy + kCpEx; t += blockDim.x) sE[t] = a.etab[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  CpBuf* bufs = reinterpret_cast<CpBuf*>(smem + kCpEtabBytes) + 2 * warp;
  const int part = lane & 1, c = (lane >> 1) % CC, grp = lane / (2 * CC);
  const int64_t nsj = a.hdr[2];
  const int64_t per = a.nbpt * a.ncc;
  const int64_t njobs = nsj * per;
  for (int64_t job = (int64_t)blockIdx.x * kCpWarps + warp; job < njobs; job += (int64_t)gridDim.x * kCpWarps) {
    const Item it = a.jobs[job / per];
    const int64_t rest = job % per;
    const int cc = (int)(rest % a.ncc);
    const int64_t bb = rest / a.ncc;
    const int64_t t = it.key / a.per_t;
    const int rem = (int)(it.key - t * a.per_t);
    const int oy = (rem / a.an1) * kCpTY, ox = (rem % a.an1) * kCpTX;
    const int ext0 = min(kCpTY, geo.K[0] - oy);
    const int64_t b = a.ntraj == 1 ? bb : t;
    const int c0 = cc * CC;
    const int ncl = (int)min((int64_t)CC, a.C - c0);
    const int64_t lbase = (int64_t)a.voff[it.key] + it.start;
    const int nent = it.len;
    const int ngr = (nent + kCpGroup - 1) / kCpGroup;

    float acc[kCpTY][kCpTX];
#pragma unroll
    for (int y = 0; y < kCpTY; ++y)
#pragma unroll
      for (int x = 0; x < kCpTX; ++x) acc[y][x] = 0.f;

    // entries one group ahead of the staging, so their loads are in flight
    // while the previous group is processed
    int4 e_cur = make_int4(0, 0, 0, 0), e_next = make_int4(0, 0, 0, 0);
    if (lane < nent) e_cur = a.vlist[lbase + lane];
    if (ngr > 1 && kCpGroup + lane < nent) e_next = a.vlist[lbase + kCpGroup + lane];
    if (ngr > 0) cp_stage<CC>(a, kdata, e_cur, lbase, min(kCpGroup, nent), lane, b, c0, ncl, bufs[0]);
    for (int q = 0; q < ngr; ++q) {
      if (q + 1 < ngr) {
        const int q1 = (q + 1) * kCpGroup;
        cp_stage<CC>(a, kdata, e_next, lbase + q1, min(kCpGroup, nent - q1), lane, b, c0, ncl, bufs[(q + 1) & 1]);
        const int q2 = q1 + kCpGroup;
        if (q2 + lane < nent) e_next = a.vlist[lbase + q2 + lane];
        cp_wait<1>();
      } else {
        cp_wait<0>();
      }
      __syncwarp();
      const CpBuf& buf = bufs[q & 1];
      const int myk = buf.meta[lane];
      const unsigned present = __reduce_or_sync(0xffffffffu, 1u << (myk & 31));
      const CpPtr base{&buf.rec[0][0], reinterpret_cast<const float2*>(&buf.rec[3][0]) + part, buf.sv + c * kCpSVS};
      cp_keys<CC, 0>(base, present, myk, 0, grp, acc);
      __syncwarp();  // the buffer is staged again two groups later
    }

    // the lane groups' tiles meet (fixed order: deterministic)
    if constexpr (G > 1) {
#pragma unroll
      for (int y = 0; y < kCpTY; ++y)
#pragma unroll
        for (int x = 0; x < kCpTX; ++x)
#pragma unroll
          for (int o = 2 * CC; o < 32; o <<= 1) acc[y][x] += __shfl_xor_sync(0xffffffffu, acc[y][x], o);
    }
    // write-out: lane part p takes cells x = 2p, 2p + 1 of each row as complex
    // values (the other part from its partner lane), times R = conj(Ey[y] Ex[x])
    const bool writer = grp == 0 && c < ncl;
    const float2 rx0 = cconj<float>(sE[kCpEy + kCpE0 + 2 * part]);
    const float2 rx1 = cconj<float>(sE[kCpEy + kCpE0 + 2 * part + 1]);
    float2* dst0 = grid + (b * a.C + c0 + c) * a.gtot + (int64_t)oy * geo.K[1] + ox + 2 * part;
#pragma unroll
    for (int y = 0; y < kCpTY; ++y) {
      const float s0 = part ? acc[y][0] : acc[y][2];
      const float s1 = part ? acc[y][1] : acc[y][3];
      const float r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
      const float r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
      float2 z0 = part ? make_float2(r0, acc[y][2]) : make_float2(acc[y][0], r0);
      float2 z1 = part ? make_float2(r1, acc[y][3]) : make_float2(acc[y][1], r1);
      if (writer && y < ext0) {
        const float2 ry = cconj<float>(sE[kCpE0 + y]);
        z0 = cmul<float>(cmul<float>(z0, ry), rx0);
        z1 = cmul<float>(cmul<float>(z1, ry), rx1);
        float2* d = dst0 + (int64_t)y * geo.K[1];
        if (it.pad) {
          atomicAdd(d, z0);
          atomicAdd(d + 1, z1);
        } else {
          *reinterpret_cast<float4*>(d) = make_float4(z0.x, z0.y, z1.x, z1.y);
        }
      }
    }
  }
}

// The entries' records, once per layout and table set (after the per-point
// linear-phase pre-pass): one thread per list entry reads its point's factors
// {mx[6], my[6], P} and writes {MX[4] = mx[x - rx]}, {my0..3}, {my4, my5, 0,
// 0}, {Q.x, -Q.y, Q.y, Q.x} with Q = P Ey[2 + ry] Ex[2 + rx] to its group's
// sorted slot. One CTA per output tile.
__global__ void __launch_bounds__(256) k_atile_records(int64_t nkeys, const int32_t* __restrict__ voff,
                                                       const int32_t* __restrict__ vcount,
                                                       const int4* __restrict__ vlist,
                                                       const float4* __restrict__ pfac,
                                                       const float2* __restrict__ etab, float4* __restrict__ arec) {
  for (int64_t key = blockIdx.x; key < nkeys; key += gridDim.x) {
    const int cnt = vcount[key];
    const int64_t base = voff[key];
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      const int4 e = vlist[base + j];
      const int ry = (e.z & 0xff) - 5, rx = ((e.z >> 8) & 0xff) - 5, rank = (e.z >> 16) & 0xff;
      const float4* src = pfac + (int64_t)e.x * 4;
      const float4 f0 = src[0], f1 = src[1], f2 = src[2], f3 = src[3];
      const float mx[6] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y};
      float MX[kCpTX];
#pragma unroll
      for (int x = 0; x < kCpTX; ++x) {
        const int jj = x - rx;
        float m = 0.f;
#pragma unroll
        for (int tt = 0; tt < 6; ++tt) m = jj == tt ? mx[tt] : m;
        MX[x] = m;
      }
      const float2 Q =
          cmul<float>(cmul<float>(make_float2(f3.x, f3.y), etab[kCpE0 + 2 + ry]), etab[kCpEy + kCpE0 + 2 + rx]);
      float4* dst = arec + (base + (j / kCpGroup) * kCpGroup + rank) * 4;
      dst[0] = make_float4(MX[0], MX[1], MX[2], MX[3]);
      dst[1] = make_float4(f1.z, f1.w, f2.x, f2.y);
      dst[2] = make_float4(f2.z, f2.w, 0.f, 0.f);
      dst[3] = make_float4(Q.x, -Q.y, Q.y, Q.x);
    }
  }
}

// Zero the output tiles split over several sub-jobs (accumulated with
// atomics), in every plane of the batch items they serve. Sub-jobs are sorted
// longest first and a split tile's first sub-job is a full kCpSubjob long.
__global__ void k_zero_split_atiles(Geo<float> geo, CpLaunch a, float2* __restrict__ grid) {
  const int64_t nsj = a.hdr[2];
  for (int64_t j = blockIdx.x; j < nsj; j += gridDim.x) {
    const Item it = a.jobs[j];
    if (it.len < kCpSubjob) break;
    if (!(it.pad && it.start == 0)) continue;
    const int64_t t = it.key / a.per_t;
    const int rem = (int)(it.key - t * a.per_t);
    const int oy = (rem / a.an1) * kCpTY, ox = (rem % a.an1) * kCpTX;
    const int ext0 = min(kCpTY, geo.K[0] - oy);
    const int64_t b0 = a.ntraj == 1 ? 0 : t, nb = a.ntraj == 1 ? a.B : 1;
    const int64_t rows = nb * a.C * ext0;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) {
      const int64_t plane = b0 * a.C + r / ext0;
      const int y = (int)(r % ext0);
      float4* d = reinterpret_cast<float4*>(grid + plane * a.gtot + (int64_t)(oy + y) * geo.K[1] + ox);
      d[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      d[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

}  // namespace tkbn

namespace tkbn_host {

using namespace tkbn;

static size_t adj_cp_smem() { return (size_t)kCpEtabBytes + (size_t)2 * kCpWarps * sizeof(CpBuf); }

bool adj_cp_eligible(const PointsLayout& L, int64_t Cc, const void* grid) {
  return L.atile && L.pfac && Cc <= 16 && (uintptr_t)grid % 16 == 0;
}

int adj_cp_records(const PointsLayout& L, const char* ws, const float2* pfac, const float2* etab, cudaStream_t s) {
  const int64_t nb = L.natile < 152 * 8 ? L.natile : 152 * 8;
  k_atile_records<<<(int)(nb < 1 ? 1 : nb), 256, 0, s>>>(
      L.natile, (const int32_t*)(ws + L.off_avoff), (const int32_t*)(ws + L.off_avcount),
      (const int4*)(ws + L.off_avlist), reinterpret_cast<const float4*>(pfac), etab,
      (float4*)const_cast<char*>(ws + L.off_arec));
  return check_cuda(cudaGetLastError(), "entry records launch");
}

int adj_cp_launch(const Geo<float>& geo, const PointsLayout& L, const char* ws, const float2* etab, int64_t M,
                  int64_t ntraj, int64_t B, int64_t C, int Cc, int ncc, int64_t nbpt, int64_t gtot,
                  const void* kdata, void* grid, cudaStream_t s) {
  CpLaunch a;
  a.jobs = (const Item*)(ws + L.off_ajobs);
  a.hdr = (const int64_t*)(ws + L.off_hdr);
  a.vlist = (const int4*)(ws + L.off_avlist);
  a.voff = (const int32_t*)(ws + L.off_avoff);
  a.arec = (const float4*)(ws + L.off_arec);
  a.etab = etab;
  a.M = M;
  a.ntraj = ntraj;
  a.B = B;
  a.C = C;
  a.ncc = ncc;
  a.nbpt = nbpt;
  a.gtot = gtot;
  a.an1 = L.antile[1];
  a.per_t = L.antile[0] * L.antile[1];
  {
    const int64_t zb = L.max_subjobs_a < 152 * 4 ? L.max_subjobs_a : 152 * 4;
    k_zero_split_atiles<<<(int)(zb < 1 ? 1 : zb), 256, 0, s>>>(geo, a, (float2*)grid);
    int rc = check_cuda(cudaGetLastError(), "zero split tiles launch");
    if (rc) return rc;
  }
  const size_t smem = adj_cp_smem();
  auto launch = [&](auto kernel) {
    int64_t per_gpu = 0;
    int rc = resident_grid((const void*)kernel, kCpWarps * 32, smem, &per_gpu);
    if (rc) return rc;
    const int64_t max_jobs = (L.max_subjobs_a * nbpt * ncc + kCpWarps - 1) / kCpWarps;
    int64_t blocks = per_gpu < max_jobs ? per_gpu : max_jobs;
    if (blocks < 1) blocks = 1;
    kernel<<<(int)blocks, kCpWarps * 32, smem, s>>>(geo, a, (const float2*)kdata, (float2*)grid);
    return check_cuda(cudaGetLastError(), "interp_adj launch");
  };
  switch (Cc) {
    case 1: return launch(k_adj_cp<1>);
    case 2: return launch(k_adj_cp<2>);
    case 4: return launch(k_adj_cp<4>);
    case 8: return launch(k_adj_cp<8>);
    case 16: return launch(k_adj_cp<16>);
    default: return set_error(TKBN_ERR_UNSUPPORTED, "coil-part adjoint: %d coils per job", Cc);
  }
}

}  // namespace tkbn_host
