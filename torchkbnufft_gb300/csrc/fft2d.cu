// K2/K5/K6 for 2D grids: the oversampled FFT written out as separable
// row and column passes, fused with the zero pad, the crop, the scaling,
// the coil-map multiply and coil sum, and (Toeplitz) the kernel multiply.
//
// Because the image occupies only rows n0 < N0 and columns n1 < N1 of the
// K0 x K1 grid, the forward transform does the row FFTs of the N0 nonzero
// rows only (fused with the pad: the image is read directly), then the
// column FFTs with the zero rows skipped on load; the inverse does the
// column FFTs keeping only the N0 rows the crop uses, then the row FFTs of
// those rows fused with the crop, the conjugate scaling and the coil sum.
// Both work in place in the caller's grid buffer. Compared with a full 2D
// FFT between separate pad and crop kernels this moves about 2.5x fewer
// bytes through HBM (and 5x fewer for the Toeplitz operator, whose column
// pass does FFT, kernel multiply and inverse FFT of each column at once).
//
// Each 1D transform is a Stockham autosort FFT in shared memory. A CTA runs
// F transforms side by side (element m of transform f at buf[m*F + f], so
// a warp's accesses in every stage cover whole 32-byte sectors and F
// neighbouring columns are one coalesced segment in global memory). Stage s
// of radix R_s does n/R_s butterflies per transform: butterfly j loads
// x[j + r n/R_s], multiplies by the twiddles w^(r k n/(Ns R_s)) with
// k = j mod Ns (Ns = product of the earlier radices, w = exp(-+2 pi i/n))
// and writes DFT_R(x) to y[(j/Ns) Ns R_s + k + r Ns]. Radices 2..15 are
// unrolled register DFTs (6, 10, 12 and 15 as prime-factor products, which
// need no inner twiddles). Twiddles come from a table exp(-2 pi i m/n)
// computed on the host in double precision.
//
// Reference semantics: fft_and_scale / ifft_and_scale / fft_filter,
// torchkbnufft/_nufft/fft.py:35-173 (torch.fft.fftn / ifftn over the last
// two dims, "ortho" = 1/sqrt(prod K) each way), with the SENSE multiply and
// coil sum of torchkbnufft/modules/kbnufft.py:182-183 and 404-405.

#include "fft2d.cuh"

#include <cmath>
#include <new>
#include <type_traits>

namespace tkbn {

// ------------------------------------------------------------ register DFTs
// Multiply by s*i (s = +1 or -1).
template <typename R, int S>
__device__ __forceinline__ cplx<R> mul_si(cplx<R> a) {
  return S > 0 ? mk<R>(-a.y, a.x) : mk<R>(a.y, -a.x);
}
template <typename R>
__device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x + b.x, a.y + b.y);
}
template <typename R>
__device__ __forceinline__ cplx<R> csub(cplx<R> a, cplx<R> b) {
  return mk<R>(a.x - b.x, a.y - b.y);
}

// Asynchronous global -> shared copy of one complex element: a thread
// issues all of its copies back to back and waits once.
__device__ __forceinline__ void cp_async_c(float2* smem_dst, const float2* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_c(double2* smem_dst, const double2* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// all committed groups but the most recent one have landed
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// y_k = sum_n x_n exp(DIR 2 pi i n k / N), in place; DIR = -1 forward.
template <typename R, int DIR, int N>
struct Dft;

template <typename R, int DIR>
struct Dft<R, DIR, 1> {
  static __device__ __forceinline__ void run(cplx<R>*) {}
};

template <typename R, int DIR>
struct Dft<R, DIR, 2> {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    const cplx<R> a = v[0], b = v[1];
    v[0] = cadd<R>(a, b);
    v[1] = csub<R>(a, b);
  }
};

template <typename R, int DIR>
struct Dft<R, DIR, 3> {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    const R h = R(0.86602540378443864676);  // sin(2 pi / 3)
    const cplx<R> t1 = cadd<R>(v[1], v[2]);
    const cplx<R> t2 = mk<R>(v[0].x - R(0.5) * t1.x, v[0].y - R(0.5) * t1.y);
    const cplx<R> d = csub<R>(v[1], v[2]);
    const cplx<R> t3 = mul_si<R, DIR>(mk<R>(h * d.x, h * d.y));
    v[0] = cadd<R>(v[0], t1);
    v[1] = cadd<R>(t2, t3);
    v[2] = csub<R>(t2, t3);
  }
};

template <typename R, int DIR>
struct Dft<R, DIR, 4> {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    const cplx<R> s02 = cadd<R>(v[0], v[2]), d02 = csub<R>(v[0], v[2]);
    const cplx<R> s13 = cadd<R>(v[1], v[3]), d13 = mul_si<R, DIR>(csub<R>(v[1], v[3]));
    v[0] = cadd<R>(s02, s13);
    v[2] = csub<R>(s02, s13);
    v[1] = cadd<R>(d02, d13);
    v[3] = csub<R>(d02, d13);
  }
};

template <typename R, int DIR>
struct Dft<R, DIR, 5> {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    // cos and sin of 2 pi / 5 and 4 pi / 5
    const R c1 = R(0.30901699437494742410), c2 = R(-0.80901699437494742410);
    const R s1 = R(0.95105651629515357212), s2 = R(0.58778525229247312917);
    const cplx<R> b1 = cadd<R>(v[1], v[4]), b2 = cadd<R>(v[2], v[3]);
    const cplx<R> d1 = csub<R>(v[1], v[4]), d2 = csub<R>(v[2], v[3]);
    const cplx<R> a0 = v[0];
    const cplx<R> r1 = mk<R>(a0.x + c1 * b1.x + c2 * b2.x, a0.y + c1 * b1.y + c2 * b2.y);
    const cplx<R> r2 = mk<R>(a0.x + c2 * b1.x + c1 * b2.x, a0.y + c2 * b1.y + c1 * b2.y);
    const cplx<R> i1 = mul_si<R, DIR>(mk<R>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
    const cplx<R> i2 = mul_si<R, DIR>(mk<R>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
    v[0] = mk<R>(a0.x + b1.x + b2.x, a0.y + b1.y + b2.y);
    v[1] = cadd<R>(r1, i1);
    v[4] = csub<R>(r1, i1);
    v[2] = cadd<R>(r2, i2);
    v[3] = csub<R>(r2, i2);
  }
};

template <typename R, int DIR>
struct Dft<R, DIR, 8> {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    const R q = R(0.70710678118654752440);  // sqrt(1/2)
    cplx<R> e[4] = {v[0], v[2], v[4], v[6]};
    cplx<R> o[4] = {v[1], v[3], v[5], v[7]};
    Dft<R, DIR, 4>::run(e);
    Dft<R, DIR, 4>::run(o);
    // o_k *= exp(DIR 2 pi i k / 8)
    o[1] = mk<R>(q * (o[1].x - DIR * o[1].y), q * (o[1].y + DIR * o[1].x));
    o[2] = mul_si<R, DIR>(o[2]);
    o[3] = mk<R>(q * (-o[3].x - DIR * o[3].y), q * (-o[3].y + DIR * o[3].x));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd<R>(e[k], o[k]);
      v[k + 4] = csub<R>(e[k], o[k]);
    }
  }
};

// Prime-factor DFT of size N1*N2 (coprime): the input index map
// n = (N2 n1 + N1 n2) mod N and the output map k -> (k mod N1, k mod N2)
// turn it into an N1 x N2 2D DFT with no inner twiddles.
template <typename R, int DIR, int N1, int N2>
struct DftPfa {
  static __device__ __forceinline__ void run(cplx<R>* v) {
    constexpr int N = N1 * N2;
    cplx<R> a[N1][N2];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1)
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) a[n1][n2] = v[(N2 * n1 + N1 * n2) % N];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) Dft<R, DIR, N2>::run(a[n1]);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      cplx<R> col[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) col[n1] = a[n1][k2];
      Dft<R, DIR, N1>::run(col);
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) a[k1][k2] = col[k1];
    }
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = a[k % N1][k % N2];
  }
};

template <typename R, int DIR>
struct Dft<R, DIR, 6> : DftPfa<R, DIR, 2, 3> {};
template <typename R, int DIR>
struct Dft<R, DIR, 10> : DftPfa<R, DIR, 2, 5> {};
template <typename R, int DIR>
struct Dft<R, DIR, 12> : DftPfa<R, DIR, 4, 3> {};
template <typename R, int DIR>
struct Dft<R, DIR, 15> : DftPfa<R, DIR, 3, 5> {};

// ------------------------------------------------------------ FFT stages
template <typename R, int DIR>
__device__ __forceinline__ cplx<R> twiddle(const cplx<R>* __restrict__ tw, int m) {
  const cplx<R> w = tw[m];
  return DIR < 0 ? w : mk<R>(w.x, -w.y);
}

template <typename R, int DIR, int RAD>
__device__ __forceinline__ void fft_stage(const cplx<R>* __restrict__ in, cplx<R>* __restrict__ out, int n, int Ns,
                                          int F, int f, int tj, int P, const cplx<R>* __restrict__ tw) {
  const int T = n / RAD;
  const int tstep = n / (Ns * RAD);
  for (int j = tj; j < T; j += P) {
    const int k = j % Ns;
    cplx<R> v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[r] = in[(j + r * T) * F + f];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < RAD; ++r) v[r] = cmul<R>(v[r], twiddle<R, DIR>(tw, r * k * tstep));
    }
    Dft<R, DIR, RAD>::run(v);
    const int base = (j - k) * RAD + k;
#pragma unroll
    for (int r = 0; r < RAD; ++r) out[(base + r * Ns) * F + f] = v[r];
  }
}

// Runs every stage of the plan on the F transforms held in buf0 (buf1 is the
// other half of the ping-pong pair); returns the buffer holding the result.
// All threads of the CTA must call it (it synchronises between stages).
template <typename R, int DIR>
__device__ cplx<R>* fft_smem(cplx<R>* buf0, cplx<R>* buf1, const FftPlan1& pl, const cplx<R>* __restrict__ tw,
                             int F, int f, int tj) {
  cplx<R>* in = buf0;
  cplx<R>* out = buf1;
  int Ns = 1;
  for (int s = 0; s < pl.nst; ++s) {
    const int rad = pl.rad[s];
    switch (rad) {
      case 2: fft_stage<R, DIR, 2>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 3: fft_stage<R, DIR, 3>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 4: fft_stage<R, DIR, 4>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 5: fft_stage<R, DIR, 5>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 6: fft_stage<R, DIR, 6>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 8: fft_stage<R, DIR, 8>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 10: fft_stage<R, DIR, 10>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      case 12: fft_stage<R, DIR, 12>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
      default: fft_stage<R, DIR, 15>(in, out, pl.n, Ns, F, f, tj, pl.P, tw); break;
    }
    __syncthreads();
    cplx<R>* t = in;
    in = out;
    out = t;
    Ns *= rad;
  }
  return in;
}

// Compile-time plans for the common grid sizes: every stride, loop bound
// and index division of the stages becomes a constant. P = threads per
// transform (the busiest stage's butterflies, a multiple of 8).
template <int N>
struct CtPlan {
  static constexpr int R0 = 1, R1 = 1, R2 = 1, R3 = 1, P = 0;
};
template <>
struct CtPlan<256> {
  static constexpr int R0 = 8, R1 = 8, R2 = 4, R3 = 1, P = 64;
};
template <>
struct CtPlan<320> {
  static constexpr int R0 = 8, R1 = 8, R2 = 5, R3 = 1, P = 64;
};
template <>
struct CtPlan<384> {
  static constexpr int R0 = 8, R1 = 8, R2 = 6, R3 = 1, P = 64;
};
template <>
struct CtPlan<512> {
  static constexpr int R0 = 8, R1 = 8, R2 = 8, R3 = 1, P = 64;
};
template <>
struct CtPlan<640> {
  static constexpr int R0 = 10, R1 = 8, R2 = 8, R3 = 1, P = 80;
};
template <>
struct CtPlan<768> {
  static constexpr int R0 = 12, R1 = 8, R2 = 8, R3 = 1, P = 96;
};
template <>
struct CtPlan<1024> {
  static constexpr int R0 = 8, R1 = 8, R2 = 4, R3 = 4, P = 128;
};

template <typename R, int DIR, int N, int RAD, int NS, int P, int F = kFftF>
__device__ __forceinline__ void stage_ct(const cplx<R>* __restrict__ in, cplx<R>* __restrict__ out, int f, int tj,
                                         const cplx<R>* __restrict__ tw) {
  constexpr int T = N / RAD, TSTEP = N / (NS * RAD), ITERS = (T + P - 1) / P;
#pragma unroll
  for (int it = 0; it < ITERS; ++it) {
    const int j = tj + it * P;
    if (T % P == 0 || j < T) {
      const int k = NS == 1 ? 0 : j % NS;
      const cplx<R>* src = in + j * F + f;
      cplx<R> v[RAD];
#pragma unroll
      for (int r = 0; r < RAD; ++r) v[r] = src[r * T * F];
      if (NS > 1) {
        const int kt = k * TSTEP;
#pragma unroll
        for (int r = 1; r < RAD; ++r) v[r] = cmul<R>(v[r], twiddle<R, DIR>(tw, r * kt));
      }
      Dft<R, DIR, RAD>::run(v);
      cplx<R>* dst = out + ((j - k) * RAD + k) * F + f;
#pragma unroll
      for (int r = 0; r < RAD; ++r) dst[r * NS * F] = v[r];
    }
  }
}

template <typename R, int DIR, int N>
__device__ __forceinline__ cplx<R>* fft_ct(cplx<R>* buf0, cplx<R>* buf1, int f, int tj,
                                           const cplx<R>* __restrict__ tw) {
  using Pl = CtPlan<N>;
  stage_ct<R, DIR, N, Pl::R0, 1, Pl::P>(buf0, buf1, f, tj, tw);
  __syncthreads();
  stage_ct<R, DIR, N, Pl::R1, Pl::R0, Pl::P>(buf1, buf0, f, tj, tw);
  __syncthreads();
  if constexpr (Pl::R2 == 1) {
    return buf0;
  } else {
    stage_ct<R, DIR, N, Pl::R2, Pl::R0 * Pl::R1, Pl::P>(buf0, buf1, f, tj, tw);
    __syncthreads();
    if constexpr (Pl::R3 == 1) {
      return buf1;
    } else {
      stage_ct<R, DIR, N, Pl::R3, Pl::R0 * Pl::R1 * Pl::R2, Pl::P>(buf1, buf0, f, tj, tw);
      __syncthreads();
      return buf0;
    }
  }
}

// NC = compile-time size (a CtPlan specialisation) or 0 for the runtime plan.
template <typename R, int DIR, int NC>
__device__ __forceinline__ cplx<R>* run_fft(cplx<R>* buf0, cplx<R>* buf1, const FftPlan1& pl,
                                            const cplx<R>* __restrict__ tw, int f, int tj) {
  if constexpr (NC == 0) {
    return fft_smem<R, DIR>(buf0, buf1, pl, tw, kFftF, f, tj);
  } else {
    return fft_ct<R, DIR, NC>(buf0, buf1, f, tj, tw);
  }
}

template <int NC>
__host__ __device__ constexpr int ct_threads() {
  return NC == 0 ? kFftMaxThreads : CtPlan<NC>::P * kFftF;
}
// resident CTAs asked of the register allocator: about 1024 threads per SM
// in single precision, half that in double (twice the registers per value)
template <int NC, typename R = float>
__host__ __device__ constexpr int ct_min_blocks() {
  return NC == 0 ? 1
                 : ((1024 / ct_threads<NC>()) / (int)(sizeof(R) / sizeof(float)) > 1
                        ? (1024 / ct_threads<NC>()) / (int)(sizeof(R) / sizeof(float))
                        : 1);
}

// ------------------------------------------------------------ kernels
// Column pass over F adjacent columns of one (b, c) plane per unit.
//   kColFwd : rows >= N0 are zero on input (written by the forward row pass
//             into rows < N0 only); forward FFT; all K0 rows written.
//   kColInv : inverse FFT of all K0 rows; rows < N0 written (the crop).
//   kColToep: forward FFT (zero rows skipped), times kernel * scale,
//             inverse FFT, rows < N0 written.
enum ColMode { kColFwd = 0, kColInv = 1, kColToep = 2 };
constexpr int kColWidth = 8;  // columns per unit of the compile-time column passes
constexpr int64_t kToepPlaneFastBytes = 32ll << 20;  // see k_fft_cols_io

// Transforms that read their first stage straight from global memory and
// write their last stage straight back (compile-time plans): four passes
// over shared memory per transform instead of eight. The caller supplies the
// element access as functors: ld(i) returns input element i (zero where the
// input is padded), st(i, v) takes output element i.
//   first stage : butterfly j takes inputs j + r N/R0
//   last stage  : butterfly j gives outputs (j - k) R + k + r Ns
template <typename R, int DIR, int N, int RAD, int P, int F, class LD>
__device__ __forceinline__ void stage_ct_first(LD ld, cplx<R>* __restrict__ out, int f, int tj) {
  constexpr int T = N / RAD, ITERS = (T + P - 1) / P;
#pragma unroll
  for (int it = 0; it < ITERS; ++it) {
    const int j = tj + it * P;
    if (T % P == 0 || j < T) {
      cplx<R> v[RAD];
#pragma unroll
      for (int r = 0; r < RAD; ++r) v[r] = ld(j + r * T);
      Dft<R, DIR, RAD>::run(v);
      cplx<R>* dst = out + j * RAD * F + f;
#pragma unroll
      for (int r = 0; r < RAD; ++r) dst[r * F] = v[r];
    }
  }
}

template <typename R, int DIR, int N, int RAD, int NS, int P, int F, class ST>
__device__ __forceinline__ void stage_ct_last(const cplx<R>* __restrict__ in, ST st, int f, int tj,
                                              const cplx<R>* __restrict__ tw) {
  constexpr int T = N / RAD, TSTEP = N / (NS * RAD), ITERS = (T + P - 1) / P;
#pragma unroll
  for (int it = 0; it < ITERS; ++it) {
    const int j = tj + it * P;
    if (T % P == 0 || j < T) {
      const int k = NS == 1 ? 0 : j % NS;
      const cplx<R>* src = in + j * F + f;
      cplx<R> v[RAD];
#pragma unroll
      for (int r = 0; r < RAD; ++r) v[r] = src[r * T * F];
      if (NS > 1) {
        const int kt = k * TSTEP;
#pragma unroll
        for (int r = 1; r < RAD; ++r) v[r] = cmul<R>(v[r], twiddle<R, DIR>(tw, r * kt));
      }
      Dft<R, DIR, RAD>::run(v);
      const int base = (j - k) * RAD + k;
#pragma unroll
      for (int r = 0; r < RAD; ++r) st(base + r * NS, v[r]);
    }
  }
}

// Whole transform. FROM_GLOBAL: the first stage reads through ld, else from
// buf0. TO_GLOBAL: the last stage writes through st (returns nullptr), else
// it stays in shared memory (the returned buffer).
template <typename R, int DIR, int N, bool FROM_GLOBAL, bool TO_GLOBAL, int FW = kFftF, class LD, class ST>
__device__ __forceinline__ cplx<R>* fft_ct_io(LD ld, ST st, cplx<R>* buf0, cplx<R>* buf1, int f, int tj,
                                              const cplx<R>* __restrict__ tw) {
  using Pl = CtPlan<N>;
  constexpr int P = Pl::P * kFftF / FW;  // threads per transform: FW transforms side by side
  constexpr int S = Pl::R3 > 1 ? 4 : 3;
  static_assert(Pl::R2 > 1, "direct-IO plans have at least three stages");
  constexpr int NS1 = Pl::R0, NS2 = Pl::R0 * Pl::R1, NS3 = Pl::R0 * Pl::R1 * Pl::R2;
  if constexpr (FROM_GLOBAL) {
    stage_ct_first<R, DIR, N, Pl::R0, P, FW>(ld, buf1, f, tj);
  } else {
    stage_ct<R, DIR, N, Pl::R0, 1, P, FW>(buf0, buf1, f, tj, tw);
  }
  __syncthreads();
  stage_ct<R, DIR, N, Pl::R1, NS1, P, FW>(buf1, buf0, f, tj, tw);
  __syncthreads();
  if constexpr (S == 4) {
    stage_ct<R, DIR, N, Pl::R2, NS2, P, FW>(buf0, buf1, f, tj, tw);
    __syncthreads();
    if constexpr (TO_GLOBAL) {
      stage_ct_last<R, DIR, N, Pl::R3, NS3, P, FW>(buf1, st, f, tj, tw);
      return nullptr;
    } else {
      stage_ct<R, DIR, N, Pl::R3, NS3, P, FW>(buf1, buf0, f, tj, tw);
      __syncthreads();
      return buf0;
    }
  } else {
    if constexpr (TO_GLOBAL) {
      stage_ct_last<R, DIR, N, Pl::R2, NS2, P, FW>(buf0, st, f, tj, tw);
      return nullptr;
    } else {
      stage_ct<R, DIR, N, Pl::R2, NS2, P, FW>(buf0, buf1, f, tj, tw);
      __syncthreads();
      return buf1;
    }
  }
}

struct NoIo {
  template <typename... A>
  __device__ __forceinline__ float2 operator()(A...) const {
    return make_float2(0.f, 0.f);
  }
};

// Resident CTAs asked of the register allocator by the column pass. With
// kColWidth columns per unit, single precision: 2 (up to 128 registers) in
// general; for 256-point columns (256 threads, 32 KB of shared memory) the
// pass is bound by global-load latency at 2 CTAs per SM, so it asks for 4
// (64 registers) in the forward and inverse modes and 3 (80 registers) in the
// Toeplitz mode, the most that compile without spills.
template <typename R, int MODE, int NC, int FW>
__host__ __device__ constexpr int cols_io_min_blocks() {
  if (FW == kFftF) return ct_min_blocks<NC, R>();
  if (sizeof(R) != 4) return 1;
  if (NC == 256) return MODE == kColToep ? 3 : 4;
  return 2;
}

// Column pass with compile-time plan NC: FW adjacent columns of one plane
// per unit (every global access is a run of FW complex values), transformed
// between global memory and two shared buffers by P * kFftF / FW threads
// per column.
template <typename R, int MODE, int NC, int FW>
__global__ void __launch_bounds__(ct_threads<NC>(), cols_io_min_blocks<R, MODE, NC, FW>())
    k_fft_cols_io(Fft2dShape s, const cplx<R>* __restrict__ tw, int64_t planes, int64_t C,
                  const cplx<R>* __restrict__ kernel, int64_t kbatch, int by_channel, R scale,
                  cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int F = FW, P = CtPlan<NC>::P * kFftF / FW;
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* buf1 = buf0 + NC * F;
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const int K1 = s.K1;
  const int64_t gtot = (int64_t)NC * K1;
  const int64_t ngrp = (K1 + F - 1) / F;
  const int64_t units = planes * ngrp;
  const int nload = MODE == kColInv ? NC : s.N0;
  const int nstore = MODE == kColFwd ? NC : s.N0;
  // A Toeplitz kernel plane larger than kToepPlaneFastBytes (a 3D kernel) is
  // read by every plane that shares it: with the planes of one column group
  // run back to back, its columns come from DRAM once and from L2 for the
  // other planes. Smaller kernels stay in L2 in either order.
  const bool plane_fast = MODE == kColToep && gtot * (int64_t)sizeof(cplx<R>) > kToepPlaneFastBytes;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t plane = plane_fast ? u % planes : u / ngrp;
    const int64_t grp = plane_fast ? u / planes : u - plane * ngrp;
    const int col = (int)grp * F + f;
    const bool cok = col < K1;
    const int64_t gplane = s.pk == s.pt ? plane : (plane / s.pk) * s.pt + plane % s.pk;
    cplx<R>* g = grid + gplane * gtot + (cok ? col : 0);
    auto ld = [&](int row) { return (cok && row < nload) ? g[(int64_t)row * K1] : mk<R>(0, 0); };
    const R osc = MODE == kColToep ? R(1) : scale;
    auto st = [&](int row, cplx<R> v) {
      if (cok && row < nstore) g[(int64_t)row * K1] = cscale<R>(v, osc);
    };
    if (MODE == kColToep) {
      cplx<R>* res = fft_ct_io<R, -1, NC, true, false, FW>(ld, NoIo{}, buf0, buf1, f, tj, tw);
      const int64_t k = kbatch == 1 ? 0 : (by_channel ? plane % C : plane / C);
      const cplx<R>* kp = kernel + k * gtot + (cok ? col : 0);
      for (int m0 = tj; m0 < NC; m0 += 4 * P) {
        cplx<R> kv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          kv[q] = (cok && m < NC) ? kp[(int64_t)m * K1] : mk<R>(0, 0);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          if (m < NC) res[m * F + f] = cscale<R>(cmul<R>(res[m * F + f], kv[q]), scale);
        }
      }
      __syncthreads();
      // second transform from res; the other buffer is its partner
      if (res == buf0)
        fft_ct_io<R, +1, NC, false, true, FW>(NoIo{}, st, buf0, buf1, f, tj, tw);
      else
        fft_ct_io<R, +1, NC, false, true, FW>(NoIo{}, st, buf1, buf0, f, tj, tw);
    } else if (MODE == kColInv) {
      fft_ct_io<R, +1, NC, true, true, FW>(ld, st, buf0, buf1, f, tj, tw);
    } else {
      fft_ct_io<R, -1, NC, true, true, FW>(ld, st, buf0, buf1, f, tj, tw);
    }
    __syncthreads();
  }
}

template <typename R, int MODE, int NC>
__global__ void __launch_bounds__(ct_threads<NC>(), ct_min_blocks<NC, R>())
    k_fft_cols(Fft2dShape s, FftPlan1 pl, const cplx<R>* __restrict__ tw, int64_t planes, int64_t C,
               const cplx<R>* __restrict__ kernel, int64_t kbatch, int by_channel, R scale,
               cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int F = kFftF;
  // three buffers: the unit's data, its ping-pong partner, and the next
  // unit's data, copied in (cp.async) while this unit is transformed
  cplx<R>* const buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int bstride = pl.n * F;
  auto bufp = [=](int i) { return buf + i * bstride; };
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const int P = NC ? CtPlan<NC>::P : pl.P;
  const int K0 = s.K0, K1 = s.K1;
  const int64_t gtot = (int64_t)K0 * K1;
  const int64_t ngrp = (K1 + F - 1) / F;
  const int64_t units = planes * ngrp;
  const int nload = MODE == kColInv ? K0 : s.N0;
  const int nstore = MODE == kColFwd ? K0 : s.N0;
  auto issue = [&](int64_t u, cplx<R>* dst) {
    if (u < units) {
      const int64_t plane = u / ngrp;
      const int col = (int)(u - plane * ngrp) * F + f;
      const cplx<R>* g = grid + plane * gtot + col;
      for (int m = tj; m < K0; m += P) {
        if (col < K1 && m < nload)
          cp_async_c(dst + m * F + f, g + (int64_t)m * K1);
        else
          dst[m * F + f] = mk<R>(0, 0);
      }
    }
    cp_async_commit();
  };
  int cur = 0;
  issue(blockIdx.x, bufp(0));
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int scr = cur == 2 ? 0 : cur + 1, nxt = scr == 2 ? 0 : scr + 1;
    issue(u + gridDim.x, bufp(nxt));
    cp_async_wait_prev();  // this unit's copies (all but the newest group)
    __syncthreads();
    const int64_t plane = u / ngrp;
    const int col = (int)(u - plane * ngrp) * F + f;
    const bool cok = col < K1;
    cplx<R>* g = grid + plane * gtot + col;
    cplx<R>* res;
    if (MODE == kColInv) {
      res = run_fft<R, +1, NC>(bufp(cur), bufp(scr), pl, tw, f, tj);
    } else {
      res = run_fft<R, -1, NC>(bufp(cur), bufp(scr), pl, tw, f, tj);
    }
    if (MODE == kColToep) {
      const int64_t k = kbatch == 1 ? 0 : (by_channel ? plane % C : plane / C);
      const cplx<R>* kp = kernel + k * gtot + col;
      for (int m0 = tj; m0 < K0; m0 += 4 * P) {
        cplx<R> kv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          kv[q] = (cok && m < K0) ? kp[(int64_t)m * K1] : mk<R>(0, 0);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          if (m < K0) res[m * F + f] = cscale<R>(cmul<R>(res[m * F + f], kv[q]), scale);
        }
      }
      __syncthreads();
      cplx<R>* other = res == bufp(cur) ? bufp(scr) : bufp(cur);
      res = run_fft<R, +1, NC>(res, other, pl, tw, f, tj);
    }
    const R sc = MODE == kColToep ? R(1) : scale;
    for (int m = tj; m < nstore; m += P)
      if (cok) g[(int64_t)m * K1] = cscale<R>(res[m * F + f], sc);
    __syncthreads();
    cur = nxt;
  }
  cp_async_wait();
}

// Forward row pass fused with the pad: unit = (b, n0 < N0). For each group
// of F coils, row n0 of image [* smaps] * scaling * scale, zero-padded to
// K1, is transformed and written to row n0 of the coil's grid plane.
template <typename R, int NC>
__global__ void __launch_bounds__(ct_threads<NC>()) k_fft_rows_pad(Fft2dShape s, FftPlan1 pl,
                                                                 const cplx<R>* __restrict__ tw, int64_t B, int64_t C,
                                                                 int64_t ci, const cplx<R>* __restrict__ image,
                                                                 const cplx<R>* __restrict__ smaps, int64_t sb,
                                                                 const cplx<R>* __restrict__ scaling, R scale,
                                                                 cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int F = kFftF;
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* buf1 = buf0 + pl.n * F;
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const int P = NC ? CtPlan<NC>::P : pl.P;
  const int N0 = s.N0, N1 = s.N1, K1 = s.K1;
  const int64_t ntot = (int64_t)N0 * N1, gtot = (int64_t)s.K0 * K1;
  const int64_t units = B * N0;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t b = u / N0;
    const int n0 = (int)(u - b * N0);
    const cplx<R>* sc = scaling ? scaling + (int64_t)n0 * N1 : nullptr;
    for (int64_t c0 = 0; c0 < C; c0 += F) {
      const int64_t c = c0 + f;
      const bool cok = c < C;
      const cplx<R>* im = image + (b * ci + (ci == 1 ? 0 : (cok ? c : 0))) * ntot + (int64_t)n0 * N1;
      const cplx<R>* sm = smaps ? smaps + ((sb == 1 ? 0 : b) * C + (cok ? c : 0)) * ntot + (int64_t)n0 * N1 : nullptr;
      // four elements per thread in flight: loads first, then the products
      for (int m0 = tj; m0 < K1; m0 += 4 * P) {
        cplx<R> a[4], bsm[4], bsc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          const bool in = cok && m < N1;
          a[q] = in ? im[m] : mk<R>(0, 0);
          bsm[q] = (in && sm) ? sm[m] : mk<R>(1, 0);
          bsc[q] = (in && sc) ? sc[m] : mk<R>(1, 0);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = m0 + q * P;
          cplx<R> v = a[q];
          if (sm) v = cmul<R>(v, bsm[q]);
          if (sc) v = cmul<R>(v, bsc[q]);
          if (m < K1) buf0[m * F + f] = cscale<R>(v, scale);
        }
      }
      __syncthreads();
      const cplx<R>* res = run_fft<R, -1, NC>(buf0, buf1, pl, tw, f, tj);
      if (cok) {
        cplx<R>* g = grid + (b * C + c) * gtot + (int64_t)n0 * K1;
        for (int m = tj; m < K1; m += P) g[m] = res[m * F + f];
      }
      __syncthreads();
    }
  }
}

// Forward row pass with compile-time plan NC = K1: the first stage reads
// image [* smaps] * scaling * scale straight from global memory (zero past
// N1), the last stage writes the grid row.
template <typename R, int NC>
__global__ void __launch_bounds__(ct_threads<NC>(), ct_min_blocks<NC, R>())
    k_fft_rows_pad_io(Fft2dShape s, const cplx<R>* __restrict__ tw, int64_t B, int64_t C, int64_t ci,
                      const cplx<R>* __restrict__ image, const cplx<R>* __restrict__ smaps, int64_t sb,
                      const cplx<R>* __restrict__ scaling, R scale, cplx<R>* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int F = kFftF;
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* buf1 = buf0 + NC * F;
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const int N0 = s.N0, N1 = s.N1;
  const int64_t ntot = (int64_t)N0 * N1, gtot = (int64_t)s.K0 * NC;
  const int64_t units = B * N0;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t b = u / N0;
    const int n0 = (int)(u - b * N0);
    const cplx<R>* sc = scaling ? scaling + (int64_t)n0 * N1 : nullptr;
    const int64_t grow = (int64_t)(n0 / s.ny) * s.ky + n0 % s.ny;  // the row's grid row
    for (int64_t c0 = 0; c0 < C; c0 += F) {
      const int64_t c = c0 + f;
      const bool cok = c < C;
      const cplx<R>* im = image + (b * ci + (ci == 1 ? 0 : (cok ? c : 0))) * ntot + (int64_t)n0 * N1;
      const cplx<R>* sm = smaps ? smaps + ((sb == 1 ? 0 : b) * C + (cok ? c : 0)) * ntot + (int64_t)n0 * N1 : nullptr;
      cplx<R>* g = grid + (b * C + (cok ? c : 0)) * gtot + grow * NC;
      auto ld = [&](int m) {
        cplx<R> v = mk<R>(0, 0);
        if (cok && m < N1) {
          v = im[m];
          if (sm) v = cmul<R>(v, sm[m]);
          if (sc) v = cmul<R>(v, sc[m]);
          v = cscale<R>(v, scale);
        }
        return v;
      };
      auto st = [&](int m, cplx<R> v) {
        if (cok) g[m] = v;
      };
      fft_ct_io<R, -1, NC, true, true>(ld, st, buf0, buf1, f, tj, tw);
      __syncthreads();
    }
  }
}

// Inverse row pass with compile-time plan NC = K1: the first stage reads the
// grid row, the last stage applies conj(scaling) * scale and either writes
// each coil's cropped row or (smaps) multiplies by conj(smaps), sums the F
// coils of a butterfly's lanes with shuffles and adds the group to a running
// coil sum (shared memory, one owner thread per element; the last group
// writes the sum). The coil sum is taken in the same order as the
// shared-memory kernel's.
template <typename R, int NC>
__global__ void __launch_bounds__(ct_threads<NC>(), ct_min_blocks<NC, R>())
    k_ifft_rows_crop_io(Fft2dShape s, const cplx<R>* __restrict__ tw, int64_t B, int64_t C,
                        const cplx<R>* __restrict__ grid, const cplx<R>* __restrict__ smaps, int64_t sb,
                        const cplx<R>* __restrict__ scaling, R scale, cplx<R>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int F = kFftF;
  static_assert((F & (F - 1)) == 0 && F <= 32, "coil group fits a warp");
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* buf1 = buf0 + NC * F;
  cplx<R>* acc = buf1 + NC * F;  // [N1] running coil sum (smaps only)
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const unsigned gmask = ((1u << F) - 1u) << ((threadIdx.x & 31) & ~(F - 1));
  const int N0 = s.N0, N1 = s.N1;
  const int64_t ntot = (int64_t)N0 * N1, gtot = (int64_t)s.K0 * NC;
  const int64_t units = B * N0;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t b = u / N0;
    const int n0 = (int)(u - b * N0);
    const cplx<R>* sc = scaling ? scaling + (int64_t)n0 * N1 : nullptr;
    const int64_t grow = (int64_t)(n0 / s.ny) * s.ky + n0 % s.ny;  // the row's grid row
    for (int64_t c0 = 0; c0 < C; c0 += F) {
      const int64_t c = c0 + f;
      const bool cok = c < C;
      const cplx<R>* g = grid + (b * C + (cok ? c : 0)) * gtot + grow * NC;
      auto ld = [&](int m) { return cok ? g[m] : mk<R>(0, 0); };
      if (smaps) {
        const cplx<R>* sm = smaps + ((sb == 1 ? 0 : b) * C + (cok ? c : 0)) * ntot + (int64_t)n0 * N1;
        cplx<R>* orow = out + b * ntot + (int64_t)n0 * N1;
        const bool first = c0 == 0, last = c0 + F >= C;
        // m is the same for the F lanes of a butterfly, so they shuffle together
        auto st = [&](int m, cplx<R> v) {
          if (m < N1) {
            cplx<R> t = mk<R>(0, 0);
            if (cok) {
              cplx<R> w = sc ? cconj<R>(sc[m]) : mk<R>(1, 0);
              w = cscale<R>(w, scale);
              t = cmul<R>(cmul<R>(v, w), cconj<R>(sm[m]));
            }
#pragma unroll
            for (int o = 1; o < F; o <<= 1) {
              t.x += __shfl_xor_sync(gmask, t.x, o);
              t.y += __shfl_xor_sync(gmask, t.y, o);
            }
            if (f == 0) {
              if (!first) t = cadd<R>(acc[m], t);
              if (last)
                orow[m] = t;
              else
                acc[m] = t;
            }
          }
        };
        fft_ct_io<R, +1, NC, true, true>(ld, st, buf0, buf1, f, tj, tw);
      } else {
        cplx<R>* orow = out + (b * C + (cok ? c : 0)) * ntot + (int64_t)n0 * N1;
        auto st = [&](int m, cplx<R> v) {
          if (cok && m < N1) {
            cplx<R> w = sc ? cconj<R>(sc[m]) : mk<R>(1, 0);
            w = cscale<R>(w, scale);
            orow[m] = cmul<R>(v, w);
          }
        };
        fft_ct_io<R, +1, NC, true, true>(ld, st, buf0, buf1, f, tj, tw);
      }
      __syncthreads();
    }
  }
}

// Inverse row pass fused with the crop: unit = (b, n0 < N0), taken in
// steps of F coils. Each step inverse transforms row n0 of F coil planes
// (the column pass left the cropped rows there); its first N1 entries times
// conj(scaling) * scale are either written per coil (no smaps) or multiplied
// by conj(smaps) and summed over coils into out[b, 0, n0, :]. The next
// step's rows are copied in (cp.async) while a step is transformed.
template <typename R, int NC>
__global__ void __launch_bounds__(ct_threads<NC>(), ct_min_blocks<NC, R>())
    k_ifft_rows_crop(Fft2dShape s, FftPlan1 pl, const cplx<R>* __restrict__ tw, int64_t B, int64_t C,
                     const cplx<R>* __restrict__ grid, const cplx<R>* __restrict__ smaps, int64_t sb,
                     const cplx<R>* __restrict__ scaling, R scale, cplx<R>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int F = kFftF;
  cplx<R>* const buf = reinterpret_cast<cplx<R>*>(smem_raw);
  const int bstride = pl.n * F;
  auto bufp = [=](int i) { return buf + i * bstride; };
  cplx<R>* acc = bufp(3);  // [N1] coil sum (smaps only)
  const int f = threadIdx.x % F, tj = threadIdx.x / F;
  const int P = NC ? CtPlan<NC>::P : pl.P;
  const int N0 = s.N0, N1 = s.N1, K1 = s.K1;
  const int64_t ntot = (int64_t)N0 * N1, gtot = (int64_t)s.K0 * K1;
  const int64_t units = B * N0;
  const int64_t ngrp = (C + F - 1) / F;
  // step t of this CTA = (unit blockIdx.x + (t / ngrp) * gridDim.x, coil group t % ngrp)
  const int64_t nsteps = units > blockIdx.x ? ((units - 1 - blockIdx.x) / gridDim.x + 1) * ngrp : 0;
  auto issue = [&](int64_t t, cplx<R>* dst) {
    if (t < nsteps) {
      const int64_t u = blockIdx.x + (t / ngrp) * gridDim.x;
      const int64_t b = u / N0;
      const int n0 = (int)(u - b * N0);
      const int64_t c = (t % ngrp) * F + f;
      const cplx<R>* g = grid + (b * C + (c < C ? c : 0)) * gtot + (int64_t)n0 * K1;
      for (int m = tj; m < K1; m += P) {
        if (c < C)
          cp_async_c(dst + m * F + f, g + m);
        else
          dst[m * F + f] = mk<R>(0, 0);
      }
    }
    cp_async_commit();
  };
  int cur = 0;
  issue(0, bufp(0));
  for (int64_t t = 0; t < nsteps; ++t) {
    const int scr = cur == 2 ? 0 : cur + 1, nxt = scr == 2 ? 0 : scr + 1;
    const int64_t u = blockIdx.x + (t / ngrp) * gridDim.x;
    const int64_t b = u / N0;
    const int n0 = (int)(u - b * N0);
    const int64_t c0 = (t % ngrp) * F;
    const int64_t c = c0 + f;
    const bool cok = c < C;
    const cplx<R>* sc = scaling ? scaling + (int64_t)n0 * N1 : nullptr;
    if (smaps && c0 == 0)
      for (int m = threadIdx.x; m < N1; m += blockDim.x) acc[m] = mk<R>(0, 0);
    issue(t + 1, bufp(nxt));
    cp_async_wait_prev();
    __syncthreads();
    const cplx<R>* res = run_fft<R, +1, NC>(bufp(cur), bufp(scr), pl, tw, f, tj);
    if (smaps) {
      const cplx<R>* sm = smaps + ((sb == 1 ? 0 : b) * C + (cok ? c : 0)) * ntot + (int64_t)n0 * N1;
      // the F coils of an element sit in F adjacent lanes: sum them with
      // shuffles, then lane f == 0 adds the group to the running sum
      for (int m0 = 0; m0 < N1; m0 += P) {
        const int m = m0 + tj;
        cplx<R> v = mk<R>(0, 0);
        if (cok && m < N1) {
          cplx<R> w = sc ? cconj<R>(sc[m]) : mk<R>(1, 0);
          w = cscale<R>(w, scale);
          v = cmul<R>(cmul<R>(res[m * F + f], w), cconj<R>(sm[m]));
        }
#pragma unroll
        for (int o = 1; o < F; o <<= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (f == 0 && m < N1) acc[m] = cadd<R>(acc[m], v);
      }
    } else if (cok) {
      cplx<R>* o = out + (b * C + c) * ntot + (int64_t)n0 * N1;
      for (int m = tj; m < N1; m += P) {
        cplx<R> w = sc ? cconj<R>(sc[m]) : mk<R>(1, 0);
        w = cscale<R>(w, scale);
        o[m] = cmul<R>(res[m * F + f], w);
      }
    }
    __syncthreads();
    if (smaps && c0 + F >= C) {
      cplx<R>* o = out + b * ntot + (int64_t)n0 * N1;
      for (int m = threadIdx.x; m < N1; m += blockDim.x) o[m] = acc[m];
      __syncthreads();
    }
    cur = nxt;
  }
  cp_async_wait();
}

}  // namespace tkbn

namespace tkbn_host {

using namespace tkbn;

// Stage radices for a transform of size n: the fewest stages (at most 4),
// then the fewest butterflies in the busiest stage.
static void search(int n, int depth, int* cur, int best_depth[1], int best_p[1], int* best) {
  static const int kRad[] = {15, 12, 10, 8, 6, 5, 4, 3, 2};
  if (n == 1) {
    int p = 0;
    for (int i = 0; i < depth; ++i) {
      int tot = 1;
      for (int k = 0; k < depth; ++k) tot *= cur[k];
      if (tot / cur[i] > p) p = tot / cur[i];
    }
    if (depth < best_depth[0] || (depth == best_depth[0] && p < best_p[0])) {
      best_depth[0] = depth;
      best_p[0] = p;
      for (int i = 0; i < depth; ++i) best[i] = cur[i];
    }
    return;
  }
  if (depth == 4) return;
  for (int r : kRad)
    if (n % r == 0) {
      cur[depth] = r;
      search(n / r, depth + 1, cur, best_depth, best_p, best);
    }
}

bool fft1_plan(int n, FftPlan1* pl) {
  if (n < 2 || n > kFftMaxN) return false;
  int cur[4], best[4], bd = 99, bp = 1 << 30;
  search(n, 0, cur, &bd, &bp, best);
  if (bd > 4) return false;
  pl->n = n;
  pl->nst = bd;
  for (int i = 0; i < 4; ++i) pl->rad[i] = i < bd ? best[i] : 1;
  // threads per transform: one per butterfly of the busiest stage, rounded
  // so that a warp holds whole groups of kFftF lanes, capped by the CTA size
  int P = bp < kFftMaxThreads / kFftF ? bp : kFftMaxThreads / kFftF;
  P = (P + 32 / kFftF - 1) / (32 / kFftF) * (32 / kFftF);
  pl->P = P;
  return true;
}

size_t fft2d_smem(const Fft2d& p, bool dbl) {
  const size_t e = dbl ? 16 : 8;
  const size_t a = 3 * (size_t)p.p0.n * kFftF * e;
  const size_t b = (3 * (size_t)p.p1.n * kFftF + p.s.N1) * e;
  return a > b ? a : b;
}

int fft1_twiddles(int n, bool dbl, void** dev) {
  const size_t bytes = (size_t)n * (dbl ? 16 : 8);
  void* host = ::operator new(bytes, std::nothrow);
  if (!host) return set_error(TKBN_ERR_INVALID, "out of host memory");
  const double pi = 3.14159265358979323846264338327950288;
  for (int m = 0; m < n; ++m) {
    // exp(-2 pi i m / n), angle reduced to [0, 2 pi) exactly in integers
    const double a = 2.0 * pi * (double)m / (double)n;
    const double cr = std::cos(a), si = -std::sin(a);
    if (dbl) {
      ((double*)host)[2 * m] = cr;
      ((double*)host)[2 * m + 1] = si;
    } else {
      ((float*)host)[2 * m] = (float)cr;
      ((float*)host)[2 * m + 1] = (float)si;
    }
  }
  int rc = check_cuda(cudaMalloc(dev, bytes), "twiddle table");
  if (!rc) rc = check_cuda(cudaMemcpy(*dev, host, bytes, cudaMemcpyHostToDevice), "twiddle upload");
  ::operator delete(host);
  return rc;
}

// Sets the kernel's shared-memory size and returns in *blocks the resident
// CTA count (SMs x CTAs per SM), capped at the number of work units.
template <typename K>
static int fft_launch_shape(K kernel, int threads, size_t smem, int64_t units, int* blocks) {
  int64_t b = 0;
  const int rc = resident_grid((const void*)kernel, threads, smem, &b);
  if (rc) return rc;
  if (units < b) b = units;
  *blocks = (int)(b < 1 ? 1 : b);
  return TKBN_OK;
}

// Calls fn(std::integral_constant<int, NC>) with NC = n when n has a
// compile-time plan, else NC = 0 (runtime plan).
template <typename R, typename Fn>
static int with_size(int n, Fn&& fn) {
  {
    switch (n) {
      case 256: return fn(std::integral_constant<int, 256>{});
      case 320: return fn(std::integral_constant<int, 320>{});
      case 384: return fn(std::integral_constant<int, 384>{});
      case 512: return fn(std::integral_constant<int, 512>{});
      case 640: return fn(std::integral_constant<int, 640>{});
      case 768: return fn(std::integral_constant<int, 768>{});
      case 1024: return fn(std::integral_constant<int, 1024>{});
      default: break;
    }
  }
  return fn(std::integral_constant<int, 0>{});
}

template <int NC>
static int threads_for(const FftPlan1& pl) {
  return (NC ? CtPlan<NC>::P : pl.P) * kFftF;
}

template <typename R, int NC>
static int cols_r(const Fft2dShape& s, const FftPlan1& pl, const void* tw, int mode, int64_t planes, int64_t C,
                  const void* kernel, int64_t kbatch, int by_channel, double scale, void* grid, cudaStream_t st) {
  if constexpr (NC != 0) {
    // compile-time plan: first and last stages straight from and to the grid,
    // kColWidth columns side by side (64-byte row runs in single precision)
    constexpr int FW = kColWidth;
    const size_t smem = 2 * (size_t)NC * FW * sizeof(cplx<R>);
    const int threads = CtPlan<NC>::P * kFftF;
    const int64_t units = planes * ((s.K1 + FW - 1) / FW);
    int blocks, rc;
    switch (mode) {
      case kColFwd:
        if ((rc = fft_launch_shape(k_fft_cols_io<R, kColFwd, NC, FW>, threads, smem, units, &blocks))) return rc;
        k_fft_cols_io<R, kColFwd, NC, FW><<<blocks, threads, smem, st>>>(s, (const cplx<R>*)tw, planes, C, nullptr,
                                                                         1, 0, (R)scale, (cplx<R>*)grid);
        break;
      case kColInv:
        if ((rc = fft_launch_shape(k_fft_cols_io<R, kColInv, NC, FW>, threads, smem, units, &blocks))) return rc;
        k_fft_cols_io<R, kColInv, NC, FW><<<blocks, threads, smem, st>>>(s, (const cplx<R>*)tw, planes, C, nullptr,
                                                                         1, 0, (R)scale, (cplx<R>*)grid);
        break;
      default:
        if ((rc = fft_launch_shape(k_fft_cols_io<R, kColToep, NC, FW>, threads, smem, units, &blocks))) return rc;
        k_fft_cols_io<R, kColToep, NC, FW><<<blocks, threads, smem, st>>>(s, (const cplx<R>*)tw, planes, C,
                                                                          (const cplx<R>*)kernel, kbatch,
                                                                          by_channel, (R)scale, (cplx<R>*)grid);
        break;
    }
    return check_cuda(cudaGetLastError(), "fft column pass launch");
  } else {
  const size_t smem = 3 * (size_t)pl.n * kFftF * sizeof(cplx<R>);
  const int threads = threads_for<NC>(pl);
  const int64_t units = planes * ((s.K1 + kFftF - 1) / kFftF);
  int blocks, rc;
  switch (mode) {
    case kColFwd:
      if ((rc = fft_launch_shape(k_fft_cols<R, kColFwd, NC>, threads, smem, units, &blocks))) return rc;
      k_fft_cols<R, kColFwd, NC><<<blocks, threads, smem, st>>>(s, pl, (const cplx<R>*)tw, planes, C, nullptr, 1, 0,
                                                           (R)scale, (cplx<R>*)grid);
      break;
    case kColInv:
      if ((rc = fft_launch_shape(k_fft_cols<R, kColInv, NC>, threads, smem, units, &blocks))) return rc;
      k_fft_cols<R, kColInv, NC><<<blocks, threads, smem, st>>>(s, pl, (const cplx<R>*)tw, planes, C, nullptr, 1, 0,
                                                           (R)scale, (cplx<R>*)grid);
      break;
    default:
      if ((rc = fft_launch_shape(k_fft_cols<R, kColToep, NC>, threads, smem, units, &blocks))) return rc;
      k_fft_cols<R, kColToep, NC><<<blocks, threads, smem, st>>>(s, pl, (const cplx<R>*)tw, planes, C,
                                                            (const cplx<R>*)kernel, kbatch, by_channel, (R)scale,
                                                            (cplx<R>*)grid);
      break;
  }
  return check_cuda(cudaGetLastError(), "fft column pass launch");
  }
}

template <typename R, int NC>
static int rows_pad_r(const Fft2dShape& s, const FftPlan1& pl, const void* tw, int64_t B, int64_t C, int64_t ci,
                      const void* image, const void* smaps, int64_t sb, const void* scaling, double scale, void* grid,
                      cudaStream_t st) {
  if constexpr (NC != 0) {
    const size_t smem = 2 * (size_t)NC * kFftF * sizeof(cplx<R>);
    const int threads = CtPlan<NC>::P * kFftF;
    int blocks;
    int rc = fft_launch_shape(k_fft_rows_pad_io<R, NC>, threads, smem, B * s.N0, &blocks);
    if (rc) return rc;
    k_fft_rows_pad_io<R, NC><<<blocks, threads, smem, st>>>(s, (const cplx<R>*)tw, B, C, ci, (const cplx<R>*)image,
                                                            (const cplx<R>*)smaps, sb, (const cplx<R>*)scaling,
                                                            (R)scale, (cplx<R>*)grid);
    return check_cuda(cudaGetLastError(), "fft row pass launch");
  } else {
    const size_t smem = 2 * (size_t)pl.n * kFftF * sizeof(cplx<R>);
    const int threads = threads_for<NC>(pl);
    int blocks;
    int rc = fft_launch_shape(k_fft_rows_pad<R, NC>, threads, smem, B * s.N0, &blocks);
    if (rc) return rc;
    k_fft_rows_pad<R, NC><<<blocks, threads, smem, st>>>(
        s, pl, (const cplx<R>*)tw, B, C, ci, (const cplx<R>*)image, (const cplx<R>*)smaps, sb,
        (const cplx<R>*)scaling, (R)scale, (cplx<R>*)grid);
    return check_cuda(cudaGetLastError(), "fft row pass launch");
  }
}

template <typename R, int NC>
static int rows_crop_r(const Fft2dShape& s, const FftPlan1& pl, const void* tw, int64_t B, int64_t C,
                       const void* grid, const void* smaps, int64_t sb, const void* scaling, double scale, void* out,
                       cudaStream_t st) {
  if constexpr (NC != 0) {
    const size_t smem = (2 * (size_t)NC * kFftF + s.N1) * sizeof(cplx<R>);
    const int threads = CtPlan<NC>::P * kFftF;
    int blocks;
    int rc = fft_launch_shape(k_ifft_rows_crop_io<R, NC>, threads, smem, B * s.N0, &blocks);
    if (rc) return rc;
    k_ifft_rows_crop_io<R, NC><<<blocks, threads, smem, st>>>(s, (const cplx<R>*)tw, B, C, (const cplx<R>*)grid,
                                                              (const cplx<R>*)smaps, sb, (const cplx<R>*)scaling,
                                                              (R)scale, (cplx<R>*)out);
    return check_cuda(cudaGetLastError(), "ifft row pass launch");
  } else {
    const size_t smem = (3 * (size_t)pl.n * kFftF + s.N1) * sizeof(cplx<R>);
    const int threads = threads_for<NC>(pl);
    int blocks;
    int rc = fft_launch_shape(k_ifft_rows_crop<R, NC>, threads, smem, B * s.N0, &blocks);
    if (rc) return rc;
    k_ifft_rows_crop<R, NC><<<blocks, threads, smem, st>>>(
        s, pl, (const cplx<R>*)tw, B, C, (const cplx<R>*)grid, (const cplx<R>*)smaps, sb, (const cplx<R>*)scaling,
        (R)scale, (cplx<R>*)out);
    return check_cuda(cudaGetLastError(), "ifft row pass launch");
  }
}

template <typename R>
static int forward_r(const Fft2d& p, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                     int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st) {
  int rc = with_size<R>(p.p1.n, [&](auto nc) {
    return rows_pad_r<R, decltype(nc)::value>(p.s, p.p1, p.tw1, B, C, ci, image, smaps, sb, scaling, scale, grid, st);
  });
  if (rc) return rc;
  return with_size<R>(p.p0.n, [&](auto nc) {
    return cols_r<R, decltype(nc)::value>(p.s, p.p0, p.tw0, kColFwd, B * C, C, nullptr, 1, 0, 1.0, grid, st);
  });
}

template <typename R>
static int inverse_r(const Fft2d& p, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                     const void* scaling, double scale, void* out, cudaStream_t st) {
  int rc = with_size<R>(p.p0.n, [&](auto nc) {
    return cols_r<R, decltype(nc)::value>(p.s, p.p0, p.tw0, kColInv, B * C, C, nullptr, 1, 0, 1.0, grid, st);
  });
  if (rc) return rc;
  return with_size<R>(p.p1.n, [&](auto nc) {
    return rows_crop_r<R, decltype(nc)::value>(p.s, p.p1, p.tw1, B, C, grid, smaps, sb, scaling, scale, out, st);
  });
}

template <typename R>
static int toeplitz_r(const Fft2d& p, int64_t B, int64_t C, int64_t ci, const void* image, const void* kernel,
                      int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale, void* grid,
                      void* out, cudaStream_t st) {
  int rc = with_size<R>(p.p1.n, [&](auto nc) {
    return rows_pad_r<R, decltype(nc)::value>(p.s, p.p1, p.tw1, B, C, ci, image, smaps, sb, nullptr, scale, grid, st);
  });
  if (rc) return rc;
  rc = with_size<R>(p.p0.n, [&](auto nc) {
    return cols_r<R, decltype(nc)::value>(p.s, p.p0, p.tw0, kColToep, B * C, C, kernel, kbatch, by_channel, scale,
                                          grid, st);
  });
  if (rc) return rc;
  return with_size<R>(p.p1.n, [&](auto nc) {
    return rows_crop_r<R, decltype(nc)::value>(p.s, p.p1, p.tw1, B, C, grid, smaps, sb, nullptr, 1.0, out, st);
  });
}

int fft2d_forward(const Fft2d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                  int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st) {
  return dtype == TKBN_C64 ? forward_r<float>(p, B, C, ci, image, smaps, sb, scaling, scale, grid, st)
                           : forward_r<double>(p, B, C, ci, image, smaps, sb, scaling, scale, grid, st);
}

int fft2d_inverse(const Fft2d& p, int dtype, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                  const void* scaling, double scale, void* out, cudaStream_t st) {
  return dtype == TKBN_C64 ? inverse_r<float>(p, B, C, grid, smaps, sb, scaling, scale, out, st)
                           : inverse_r<double>(p, B, C, grid, smaps, sb, scaling, scale, out, st);
}

static bool ct_size(int n) {
  return n == 256 || n == 320 || n == 384 || n == 512 || n == 640 || n == 768 || n == 1024;
}

bool fft3d_supported(const int K[3]) { return ct_size(K[0]) && ct_size(K[1]) && ct_size(K[2]); }

// Shapes of the three passes of a 3D transform: the x rows of the nonzero
// (z, y) image rows, the y columns of the nonzero z slices, and the z columns
// of each volume seen as Kz rows of Ky*Kx columns.
static Fft2dShape rows3(const Fft3d& p) {
  Fft2dShape s = fft2d_shape(p.N[0] * p.N[1], p.N[2], p.K[0] * p.K[1], p.K[2]);
  s.ny = p.N[1];
  s.ky = p.K[1];
  return s;
}
static Fft2dShape cols_y3(const Fft3d& p) {
  Fft2dShape s = fft2d_shape(p.N[1], p.N[2], p.K[1], p.K[2]);
  s.pk = p.N[0];
  s.pt = p.K[0];
  return s;
}
static Fft2dShape cols_z3(const Fft3d& p) { return fft2d_shape(p.N[0], p.N[1] * p.N[2], p.K[0], p.K[1] * p.K[2]); }

static const FftPlan1 kNoPlan = {0, 0, {0, 0, 0, 0}, 0};

template <typename R>
static int forward3_r(const Fft3d& p, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                      int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st) {
  int rc = with_size<R>(p.K[2], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return rows_pad_r<R, decltype(nc)::value>(rows3(p), kNoPlan, p.tw[2], B, C, ci, image, smaps, sb, scaling,
                                                scale, grid, st);
    }
  });
  if (rc) return rc;
  rc = with_size<R>(p.K[1], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return cols_r<R, decltype(nc)::value>(cols_y3(p), kNoPlan, p.tw[1], kColFwd, B * C * p.N[0], C, nullptr, 1, 0,
                                            1.0, grid, st);
    }
  });
  if (rc) return rc;
  return with_size<R>(p.K[0], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return cols_r<R, decltype(nc)::value>(cols_z3(p), kNoPlan, p.tw[0], kColFwd, B * C, C, nullptr, 1, 0, 1.0,
                                            grid, st);
    }
  });
}

template <typename R>
static int inverse3_r(const Fft3d& p, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                      const void* scaling, double scale, void* out, cudaStream_t st) {
  int rc = with_size<R>(p.K[0], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return cols_r<R, decltype(nc)::value>(cols_z3(p), kNoPlan, p.tw[0], kColInv, B * C, C, nullptr, 1, 0, 1.0,
                                            grid, st);
    }
  });
  if (rc) return rc;
  rc = with_size<R>(p.K[1], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return cols_r<R, decltype(nc)::value>(cols_y3(p), kNoPlan, p.tw[1], kColInv, B * C * p.N[0], C, nullptr, 1, 0,
                                            1.0, grid, st);
    }
  });
  if (rc) return rc;
  return with_size<R>(p.K[2], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes");
    } else {
      return rows_crop_r<R, decltype(nc)::value>(rows3(p), kNoPlan, p.tw[2], B, C, grid, smaps, sb, scaling, scale,
                                                 out, st);
    }
  });
}

int fft3d_forward(const Fft3d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image, const void* smaps,
                  int64_t sb, const void* scaling, double scale, void* grid, cudaStream_t st) {
  return dtype == TKBN_C64 ? forward3_r<float>(p, B, C, ci, image, smaps, sb, scaling, scale, grid, st)
                           : forward3_r<double>(p, B, C, ci, image, smaps, sb, scaling, scale, grid, st);
}

int fft3d_inverse(const Fft3d& p, int dtype, int64_t B, int64_t C, void* grid, const void* smaps, int64_t sb,
                  const void* scaling, double scale, void* out, cudaStream_t st) {
  return dtype == TKBN_C64 ? inverse3_r<float>(p, B, C, grid, smaps, sb, scaling, scale, out, st)
                           : inverse3_r<double>(p, B, C, grid, smaps, sb, scaling, scale, out, st);
}

// Toeplitz filter on a 3D grid: x rows and y columns forward, the z columns
// transformed, multiplied by the kernel and transformed back in one pass,
// then y columns and x rows inverse (with the crop and coil sum).
template <typename R>
static int toeplitz3_r(const Fft3d& p, int64_t B, int64_t C, int64_t ci, const void* image, const void* kernel,
                       int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale, void* grid,
                       void* out, cudaStream_t st) {
  auto need_ct = [] { return set_error(TKBN_ERR_UNSUPPORTED, "3D fused FFT needs compile-time plan sizes"); };
  int rc = with_size<R>(p.K[2], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return need_ct();
    } else {
      return rows_pad_r<R, decltype(nc)::value>(rows3(p), kNoPlan, p.tw[2], B, C, ci, image, smaps, sb, nullptr,
                                                scale, grid, st);
    }
  });
  if (rc) return rc;
  rc = with_size<R>(p.K[1], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return need_ct();
    } else {
      return cols_r<R, decltype(nc)::value>(cols_y3(p), kNoPlan, p.tw[1], kColFwd, B * C * p.N[0], C, nullptr, 1, 0,
                                            1.0, grid, st);
    }
  });
  if (rc) return rc;
  rc = with_size<R>(p.K[0], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return need_ct();
    } else {
      return cols_r<R, decltype(nc)::value>(cols_z3(p), kNoPlan, p.tw[0], kColToep, B * C, C, kernel, kbatch,
                                            by_channel, scale, grid, st);
    }
  });
  if (rc) return rc;
  rc = with_size<R>(p.K[1], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return need_ct();
    } else {
      return cols_r<R, decltype(nc)::value>(cols_y3(p), kNoPlan, p.tw[1], kColInv, B * C * p.N[0], C, nullptr, 1, 0,
                                            1.0, grid, st);
    }
  });
  if (rc) return rc;
  return with_size<R>(p.K[2], [&](auto nc) {
    if constexpr (decltype(nc)::value == 0) {
      return need_ct();
    } else {
      return rows_crop_r<R, decltype(nc)::value>(rows3(p), kNoPlan, p.tw[2], B, C, grid, smaps, sb, nullptr, 1.0,
                                                 out, st);
    }
  });
}

int fft3d_toeplitz(const Fft3d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image,
                   const void* kernel, int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale,
                   void* grid, void* out, cudaStream_t st) {
  return dtype == TKBN_C64
             ? toeplitz3_r<float>(p, B, C, ci, image, kernel, kbatch, by_channel, smaps, sb, scale, grid, out, st)
             : toeplitz3_r<double>(p, B, C, ci, image, kernel, kbatch, by_channel, smaps, sb, scale, grid, out, st);
}

int fft2d_toeplitz(const Fft2d& p, int dtype, int64_t B, int64_t C, int64_t ci, const void* image,
                   const void* kernel, int64_t kbatch, int by_channel, const void* smaps, int64_t sb, double scale,
                   void* grid, void* out, cudaStream_t st) {
  return dtype == TKBN_C64
             ? toeplitz_r<float>(p, B, C, ci, image, kernel, kbatch, by_channel, smaps, sb, scale, grid, out, st)
             : toeplitz_r<double>(p, B, C, ci, image, kernel, kbatch, by_channel, smaps, sb, scale, grid, out, st);
}

}  // namespace tkbn_host
