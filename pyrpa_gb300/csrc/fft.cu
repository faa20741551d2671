// Mixed-radix Stockham FFT passes in shared memory (see fft.cuh).
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdlib>
#include <string>
#include <tuple>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "fft.cuh"

namespace pgb {

namespace {

constexpr size_t kLongSmem = 200 * 1024;  // shared memory of one long-pass CTA at most

// tab[t] = exp(-2 pi i t / L); sign < 0 uses it as is, sign > 0 its conjugate
template <typename R>
__device__ __forceinline__ cx<R> twid(const cx<R>* tab, int t, int sign) {
  cx<R> w = __ldg(tab + t);
  return cmk<R>(w.x, sign < 0 ? w.y : -w.y);
}
template <typename R> __device__ __forceinline__ const cx<R>* line_tab(const PassDesc& d);
template <> __device__ __forceinline__ const double2* line_tab<double>(const PassDesc& d) { return d.tw_line; }
template <> __device__ __forceinline__ const float2* line_tab<float>(const PassDesc& d) { return d.tw_line_f; }
template <typename R> __device__ __forceinline__ const cx<R>* full_tab(const PassDesc& d);
template <> __device__ __forceinline__ const double2* full_tab<double>(const PassDesc& d) { return d.tw_full; }
template <> __device__ __forceinline__ const float2* full_tab<float>(const PassDesc& d) { return d.tw_full_f; }
template <> __device__ __forceinline__ const cdf* line_tab<dfl>(const PassDesc& d) { return d.tw_line_d; }
template <typename R> __device__ __forceinline__ const cx<R>* line_tab_y(const PassDesc& d);
template <> __device__ __forceinline__ const double2* line_tab_y<double>(const PassDesc& d) { return d.tw_line_y; }
template <> __device__ __forceinline__ const float2* line_tab_y<float>(const PassDesc& d) { return d.tw_line_y_f; }
template <> __device__ __forceinline__ const cdf* line_tab_y<dfl>(const PassDesc& d) { return d.tw_line_y_d; }
template <> __device__ __forceinline__ const cdf* full_tab<dfl>(const PassDesc& d) { return d.tw_full_d; }
// double-float roots: one 16-byte read-only load {re.hi, re.lo, im.hi, im.lo}
template <> __device__ __forceinline__ cdf twid<dfl>(const cdf* tab, int t, int sign) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(tab + t));
  return mkc(dfl(v.x, v.y), sign < 0 ? dfl(v.z, v.w) : dfl(-v.z, -v.w));
}

// Butterfly sums.  For float and double the plain sum.  For double-float the
// sum of the high words by two-sum plus the low words, without the final
// renormalization (8 flops instead of Dekker's 11): the radix-4 and radix-8
// butterflies chain two or three of these and renormalize their outputs
// once (bnorm).  Within a butterfly the low word stays a few units in the
// last place of the high word, so the normwise error stays a few 2^-47
// (|a| + |b|), as for the renormalized sum.
__device__ __forceinline__ float2 badd(float2 a, float2 b) { return a + b; }
__device__ __forceinline__ float2 bsub(float2 a, float2 b) { return a - b; }
__device__ __forceinline__ float2 bnorm(float2 a) { return a; }
__device__ __forceinline__ double2 badd(double2 a, double2 b) { return a + b; }
__device__ __forceinline__ double2 bsub(double2 a, double2 b) { return a - b; }
__device__ __forceinline__ double2 bnorm(double2 a) { return a; }
__device__ __forceinline__ dfl lazy_add(dfl a, dfl b) {
  const dfl s = two_sum(a.hi, b.hi);
  return dfl(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ cdf badd(cdf a, cdf b) { return mkc(lazy_add(a.x, b.x), lazy_add(a.y, b.y)); }
__device__ __forceinline__ cdf bsub(cdf a, cdf b) { return mkc(lazy_add(a.x, -b.x), lazy_add(a.y, -b.y)); }
__device__ __forceinline__ cdf bnorm(cdf a) {
  return mkc(fast_two_sum(a.x.hi, a.x.lo), fast_two_sum(a.y.hi, a.y.lo));
}

template <typename R, int RAD> struct Dft {
  // generic radix: direct O(RAD^2) evaluation with roots from the line table
  __device__ static void run(cx<R>* v, int sign, const cx<R>* tab, int L) {
    cx<R> o[RAD];
    const int step = L / RAD;
#pragma unroll
    for (int k = 0; k < RAD; ++k) {
      cx<R> acc = v[0];
#pragma unroll
      for (int r = 1; r < RAD; ++r) acc += v[r] * twid<R>(tab, ((r * k) % RAD) * step, sign);
      o[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < RAD; ++k) v[k] = o[k];
  }
};

template <typename R> struct Dft<R, 2> {
  __device__ static void run(cx<R>* v, int, const cx<R>*, int) {
    cx<R> a = v[0] + v[1], b = v[0] - v[1];
    v[0] = a;
    v[1] = b;
  }
};

template <typename R> struct Dft<R, 4> {
  // outputs left unrenormalized (the radix-8 butterfly goes on with them)
  __device__ static void run_lazy(cx<R>* v, int sign) {
    cx<R> a0 = badd(v[0], v[2]), a1 = bsub(v[0], v[2]), a2 = badd(v[1], v[3]);
    cx<R> a3 = muli(bsub(v[1], v[3]), (R)sign);
    v[0] = badd(a0, a2);
    v[1] = badd(a1, a3);
    v[2] = bsub(a0, a2);
    v[3] = bsub(a1, a3);
  }
  __device__ static void run(cx<R>* v, int sign, const cx<R>*, int) {
    run_lazy(v, sign);
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = bnorm(v[k]);
  }
};

template <typename R> struct Dft<R, 3> {
  __device__ static void run(cx<R>* v, int sign, const cx<R>*, int) {
    const R h = (R)0.86602540378443864676372317075294;  // sqrt(3)/2
    cx<R> t1 = v[1] + v[2], t2 = v[1] - v[2];
    cx<R> m = v[0] - (R)0.5 * t1;
    cx<R> u = h * muli(t2, (R)sign);
    v[0] = v[0] + t1;
    v[1] = m + u;
    v[2] = m - u;
  }
};

template <typename R> struct Dft<R, 5> {
  __device__ static void run(cx<R>* v, int sign, const cx<R>*, int) {
    const R c1 = (R)0.30901699437494742410229341718282;   // cos(2 pi/5)
    const R c2 = (R)-0.80901699437494742410229341718282;  // cos(4 pi/5)
    const R s1 = (R)0.95105651629515357211643933337938;   // sin(2 pi/5)
    const R s2 = (R)0.58778525229247312916870595463907;   // sin(4 pi/5)
    cx<R> a1 = v[1] + v[4], b1 = v[1] - v[4], a2 = v[2] + v[3], b2 = v[2] - v[3];
    cx<R> p1 = v[0] + c1 * a1 + c2 * a2, p2 = v[0] + c2 * a1 + c1 * a2;
    cx<R> q1 = muli(s1 * b1 + s2 * b2, (R)sign), q2 = muli(s2 * b1 - s1 * b2, (R)sign);
    v[0] = v[0] + a1 + a2;
    v[1] = p1 + q1;
    v[4] = p1 - q1;
    v[2] = p2 + q2;
    v[3] = p2 - q2;
  }
};

template <typename R> struct Dft<R, 8> {
  __device__ static void run(cx<R>* v, int sign, const cx<R>* t, int L) {
    const R h = (R)0.70710678118654752440084436210485;
    cx<R> e[4] = {v[0], v[2], v[4], v[6]};
    cx<R> o[4] = {v[1], v[3], v[5], v[7]};
    Dft<R, 4>::run_lazy(e, sign);
    Dft<R, 4>::run_lazy(o, sign);
    const R s = (R)sign;
    // o1 = o[1] (h + i s h), o3 = o[3] (-h + i s h): a sum and a difference
    // times h instead of a full complex product (fewer double-word operations)
    const cx<R> a1 = o[1], a3 = o[3];
    cx<R> o1, o3;
    if (sign > 0) {
      o1 = h * cmk<R>(a1.x - a1.y, a1.x + a1.y);
      o3 = h * cmk<R>(-(a3.x + a3.y), a3.x - a3.y);
    } else {
      o1 = h * cmk<R>(a1.x + a1.y, a1.y - a1.x);
      o3 = h * cmk<R>(a3.y - a3.x, -(a3.x + a3.y));
    }
    const cx<R> o2 = muli(o[2], s);
    v[0] = bnorm(badd(e[0], o[0]));
    v[4] = bnorm(bsub(e[0], o[0]));
    v[1] = bnorm(badd(e[1], o1));
    v[5] = bnorm(bsub(e[1], o1));
    v[2] = bnorm(badd(e[2], o2));
    v[6] = bnorm(bsub(e[2], o2));
    v[3] = bnorm(badd(e[3], o3));
    v[7] = bnorm(bsub(e[3], o3));
  }
};

// One Stockham stage (Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors", SC08, Fig. 2) over nl lines in smem.
template <typename R, int RAD>
__device__ void stage(const cx<R>* in, cx<R>* out, int L, int Ns, int nl, int sign,
                      const cx<R>* tab) {
  const int nbf = L / RAD;
  const int total = nl * nbf;
  const int tstride = L / (Ns * RAD);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int b = idx / nbf;
    const int j = idx - b * nbf;
    const cx<R>* li = in + (size_t)b * L;
    cx<R>* lo = out + (size_t)b * L;
    const int jj = j % Ns;
    cx<R> v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) {
      v[r] = li[j + r * nbf];
      if (r > 0 && jj > 0) v[r] = v[r] * twid<R>(tab, r * jj * tstride, sign);
    }
    Dft<R, RAD>::run(v, sign, tab, L);
    const int idxD = (j / Ns) * Ns * RAD + jj;
#pragma unroll
    for (int r = 0; r < RAD; ++r) lo[idxD + r * Ns] = v[r];
  }
}

// The same stage over nl lines whose line b starts at b * ls and whose
// element j sits at j * es (the plane pass's rows and columns).
template <typename R, int RAD>
__device__ void stage_strided(const cx<R>* in, cx<R>* out, int L, int Ns, int nl, int es, int ls, int sign,
                              const cx<R>* tab) {
  const int nbf = L / RAD;
  const int total = nl * nbf;
  const int tstride = L / (Ns * RAD);
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int b = idx / nbf;
    const int j = idx - b * nbf;
    const cx<R>* li = in + (size_t)b * ls;
    cx<R>* lo = out + (size_t)b * ls;
    const int jj = j % Ns;
    cx<R> v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) {
      v[r] = li[(size_t)(j + r * nbf) * es];
      if (r > 0 && jj > 0) v[r] = v[r] * twid<R>(tab, r * jj * tstride, sign);
    }
    Dft<R, RAD>::run(v, sign, tab, L);
    const int idxD = (j / Ns) * Ns * RAD + jj;
#pragma unroll
    for (int r = 0; r < RAD; ++r) lo[(size_t)(idxD + r * Ns) * es] = v[r];
  }
}

// All stages of one axis of the plane, ping-ponging in/out (swapped on return
// so that `in` holds the result).
template <typename R>
__device__ void plane_axis(cx<R>*& in, cx<R>*& out, int L, int nl, int es, int ls, int nst, const int* radix,
                           int sign, const cx<R>* tab) {
  int Ns = 1;
  for (int st = 0; st < nst; ++st) {
    const int rad = radix[st];
    switch (rad) {
      case 2: stage_strided<R, 2>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 3: stage_strided<R, 3>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 4: stage_strided<R, 4>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 5: stage_strided<R, 5>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 7: stage_strided<R, 7>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 8: stage_strided<R, 8>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 11: stage_strided<R, 11>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      case 13: stage_strided<R, 13>(in, out, L, Ns, nl, es, ls, sign, tab); break;
      default: break;
    }
    __syncthreads();
    cx<R>* t = in;
    in = out;
    out = t;
    Ns *= rad;
  }
}

// x and y axes of one (x, y) plane per CTA: the plane is read once
// (contiguous), transformed along its rows (stride 1) and columns (stride
// nx + 1, the padded row length) in shared memory, and written once.
template <typename R>
__global__ void __launch_bounds__(256) fft_plane_kernel(cx<R>* data, long long P, PassDesc d, int sign) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = d.L, ny = d.ny, sx = nx + 1, n = nx * ny;
  cx<R>* in = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* out = in + (size_t)ny * sx;
  cx<R>* arr = data + (long long)blockIdx.y * P + (long long)blockIdx.x * n;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int y = e / nx, x = e - y * nx;
    in[y * sx + x] = arr[e];
  }
  __syncthreads();
  plane_axis<R>(in, out, nx, ny, 1, sx, d.nst, d.radix, sign, line_tab<R>(d));
  plane_axis<R>(in, out, ny, nx, sx, 1, d.nst_y, d.radix_y, sign, line_tab_y<R>(d));
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int y = e / nx, x = e - y * nx;
    arr[e] = in[y * sx + x];
  }
}

// One step of the long pass: length-G^2 DFTs of nl * ntask lines of shared
// memory, done in place by groups of G threads.  Line c of line set b has its
// elements at b * LS + c * cstride + i * estride.  Thread j of a group reads
// the elements G i + j, runs a radix-G DFT over i, multiplies by w_L^(j kA)
// and writes back the slots it read; thread kA then reads G kA + j, runs a
// radix-G DFT over j and writes frequency kA + G kB (times w_M^(c k) when
// tw_out).  The trip count is the same for every thread, so that all of
// them reach each barrier.
template <typename R, int G>
__device__ void long_step(cx<R>* buf, int nl, int ntask, int LS, int cstride, int estride, int sign,
                          const cx<R>* tabL, const cx<R>* tabM, bool tw_out) {
  constexpr int L = G * G;
  const int ngroups = blockDim.x / G;
  const int group = threadIdx.x / G, lane = threadIdx.x - group * G;
  const int total = nl * ntask;
  for (int t0 = 0; t0 < total; t0 += ngroups) {
    const int task = t0 + group;
    const bool act = group < ngroups && task < total;
    int base = 0, c = 0;
    if (act) {
      const int b = task / ntask;
      c = task - b * ntask;
      base = b * LS + c * cstride;
    }
    cx<R> v[G];
    if (act) {
#pragma unroll
      for (int i = 0; i < G; ++i) v[i] = buf[base + estride * (G * i + lane)];
      Dft<R, G>::run(v, sign, tabL, L);
#pragma unroll
      for (int k = 1; k < G; ++k)
        if (lane) v[k] = v[k] * twid<R>(tabL, lane * k, sign);
#pragma unroll
      for (int k = 0; k < G; ++k) buf[base + estride * (G * k + lane)] = v[k];
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int j = 0; j < G; ++j) v[j] = buf[base + estride * (G * lane + j)];
      Dft<R, G>::run(v, sign, tabL, L);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int kb = 0; kb < G; ++kb) {
        const int k = lane + G * kb;
        cx<R> val = v[kb];
        if (tw_out) {
          const int t = c * k;  // c < L_other and k < L, so t < M
          if (t) val = val * twid<R>(tabM, t, sign);
        }
        buf[base + estride * k] = val;
      }
    }
  }
}

// A four-step axis of length M = L1 L2 (L1 = G1^2, L2 = G2^2) in one pass:
// B adjacent lines (consecutive positions at stride 1, elements at stride S)
// per CTA, each stored as L1 rows of L2 elements padded to L2 + 1.
// Forward: columns (DFT over n1, twiddle w_M^(n2 k1)), then rows (over n2);
// frequency k1 + L1 k2 ends in row k1, column k2.  Backward: rows (twiddle
// w_M^(k1 n2)), then columns.
template <typename R, int G1, int G2>
__global__ void __launch_bounds__(256) fft_long_kernel(cx<R>* data, long long P, PassDesc d, int sign) {
  constexpr int L1 = G1 * G1, L2 = G2 * G2, M = L1 * L2, RS = L2 + 1, LS = L1 * RS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* arr = data + (long long)blockIdx.y * P;
  const long long nsb = (d.S + d.B - 1) / d.B;
  const long long o = blockIdx.x / nsb;
  const long long s0 = (blockIdx.x - o * nsb) * d.B;
  const int nl = (int)min((long long)d.B, d.S - s0);
  const long long base = o * (long long)M * d.S + s0;
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int p = e / nl, b = e - p * nl;
    buf[b * LS + (p / L2) * RS + (p % L2)] = arr[base + (long long)p * d.S + b];
  }
  __syncthreads();
  const cx<R>* t1 = line_tab<R>(d);
  const cx<R>* t2 = line_tab_y<R>(d);
  const cx<R>* tm = full_tab<R>(d);
  if (sign < 0) {
    long_step<R, G1>(buf, nl, L2, LS, 1, RS, sign, t1, tm, true);   // columns n2: over n1
    __syncthreads();
    long_step<R, G2>(buf, nl, L1, LS, RS, 1, sign, t2, tm, false);  // rows k1: over n2
  } else {
    long_step<R, G2>(buf, nl, L1, LS, RS, 1, sign, t2, tm, true);   // rows k1: over k2
    __syncthreads();
    long_step<R, G1>(buf, nl, L2, LS, 1, RS, sign, t1, tm, false);  // columns n2: over k1
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int p = e / nl, b = e - p * nl;
    arr[base + (long long)p * d.S + b] = buf[b * LS + (p / L2) * RS + (p % L2)];
  }
}

template <typename R, int G1, int G2>
void launch_long_one(const PassDesc& d, dim3 grid, size_t smem, cudaStream_t s, cx<R>* data, long long P, int sign) {
  PGB_SMEM_LIMIT_ONCE((fft_long_kernel<R, G1, G2>), kLongSmem);
  fft_long_kernel<R, G1, G2><<<grid, 256, smem, s>>>(data, P, d, sign);
}

template <typename R>
void launch_long(const PassDesc& d, dim3 grid, size_t smem, cudaStream_t s, cx<R>* data, long long P, int sign) {
  if (d.lp_L1 == 64 && d.lp_L2 == 64) return launch_long_one<R, 8, 8>(d, grid, smem, s, data, P, sign);
  if (d.lp_L1 == 16 && d.lp_L2 == 64) return launch_long_one<R, 4, 8>(d, grid, smem, s, data, P, sign);
  if (d.lp_L1 == 64 && d.lp_L2 == 16) return launch_long_one<R, 8, 4>(d, grid, smem, s, data, P, sign);
  if (d.lp_L1 == 16 && d.lp_L2 == 16) return launch_long_one<R, 4, 4>(d, grid, smem, s, data, P, sign);
  throw Error("no long-pass kernel for this axis split");
}

template <typename R>
__device__ void four_step_twiddle(cx<R>* buf, const PassDesc& d, long long o, bool contig, int nl,
                                  int sign) {
  const int L = d.L;
  for (int e = threadIdx.x; e < nl * L; e += blockDim.x) {
    const int b = e / L, p = e - b * L;
    // p < L2 and k1 < L1, so p * k1 < L1 * L2 = Lfull: no reduction needed
    const long long k1 = ((contig ? o + b : o) % d.tw_L1);
    const int t = (int)((long long)p * k1);
    if (t) buf[e] = buf[e] * twid<R>(full_tab<R>(d), t, sign);
  }
}

template <typename R>
__global__ void __launch_bounds__(256) fft_pass_kernel(cx<R>* data, long long P, PassDesc d,
                                                       int sign) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* buf0 = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* buf1 = buf0 + (size_t)d.B * d.L;
  const int L = d.L;
  cx<R>* arr = data + (long long)blockIdx.y * P;
  const long long tile = blockIdx.x;
  const bool contig = (d.S == 1);
  long long o, base;
  int nl;
  if (contig) {
    const long long line0 = tile * d.B;
    nl = (int)min((long long)d.B, d.O - line0);
    base = line0 * L;
    o = line0;
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) buf0[e] = arr[base + e];
  } else {
    const long long nsb = (d.S + d.B - 1) / d.B;
    o = tile / nsb;
    const long long s0 = (tile - o * nsb) * d.B;
    nl = (int)min((long long)d.B, d.S - s0);
    base = o * L * d.S + s0;
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) {
      const int p = e / nl, b = e - p * nl;
      buf0[b * L + p] = arr[base + (long long)p * d.S + b];
    }
  }
  __syncthreads();
  if (d.tw_L1 > 0 && !d.tw_post) {
    four_step_twiddle<R>(buf0, d, o, contig, nl, sign);
    __syncthreads();
  }
  cx<R>* in = buf0;
  cx<R>* out = buf1;
  int Ns = 1;
  for (int st = 0; st < d.nst; ++st) {
    const int rad = d.radix[st];
    switch (rad) {
      case 2: stage<R, 2>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 3: stage<R, 3>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 4: stage<R, 4>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 5: stage<R, 5>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 7: stage<R, 7>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 8: stage<R, 8>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 11: stage<R, 11>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      case 13: stage<R, 13>(in, out, L, Ns, nl, sign, line_tab<R>(d)); break;
      default: break;
    }
    __syncthreads();
    cx<R>* tmp = in;
    in = out;
    out = tmp;
    Ns *= rad;
  }
  if (d.tw_L1 > 0 && d.tw_post) {
    four_step_twiddle<R>(in, d, o, contig, nl, sign);
    __syncthreads();
  }
  if (contig) {
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) arr[base + e] = in[e];
  } else {
    for (int e = threadIdx.x; e < nl * L; e += blockDim.x) {
      const int p = e / nl, b = e - p * nl;
      arr[base + (long long)p * d.S + b] = in[b * L + p];
    }
  }
}


// Two-level register FFT of lines L = A*B (see fft.cuh).  Input index
// p = B*n1 + n2, output index q = k1 + A*k2:
//   X[q] = sum_n2 w_B^(n2 k2) w_L^(n2 k1) sum_n1 w_A^(n1 k1) x[p].
template <typename R, int A, int B>
__global__ void __launch_bounds__(256) fft2_kernel(cx<R>* data, long long P, PassDesc d, int sign) {
  constexpr int L = A * B;
  constexpr int LDB = B + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* sm = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* arr = data + (long long)blockIdx.y * P;
  const long long tile = blockIdx.x;
  const bool contig = (d.S == 1);
  const int nl = d.B;
  long long o, base;
  int nact;
  if (contig) {
    const long long line0 = tile * nl;
    nact = (int)min((long long)nl, d.O - line0);
    base = line0 * L;
    o = line0;
  } else {
    const long long nsb = (d.S + nl - 1) / nl;
    o = tile / nsb;
    const long long s0 = (tile - o * nsb) * nl;
    nact = (int)min((long long)nl, d.S - s0);
    base = o * L * d.S + s0;
  }
  const bool tw4 = d.tw_L1 > 0;
  // exchange buffer: contiguous lines keep each line's row padded to B + 1
  // (threads walk n2, then lines); strided passes put the line innermost,
  // [k1][n2][line], because there adjacent threads take adjacent lines and a
  // line-outer layout would put a warp's accesses 2 (A B + A) words apart,
  // into two banks
  auto slot = [&](int b, int k1, int n2) {
    return contig ? (b * A + k1) * LDB + n2 : (k1 * B + n2) * nl + b;
  };
  // phase 1: load A elements per (line, n2), DFT over n1, inner twiddle
  for (int it = threadIdx.x; it < nl * B; it += blockDim.x) {
    int b, n2;
    if (contig) { n2 = it % B; b = it / B; } else { b = it % nl; n2 = it / nl; }
    if (b >= nact) continue;
    cx<R> v[A];
    // four-step twiddle exponent p * k1: p < L2 and k1 < L1, so the product is
    // below Lfull = L1 * L2 and indexes the table without a reduction
    const int k1o = tw4 ? (int)((contig ? o + b : o) % d.tw_L1) : 0;
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) {
      const int p = B * n1 + n2;
      const long long addr = contig ? base + (long long)b * L + p : base + (long long)p * d.S + b;
      v[n1] = arr[addr];
      if (tw4 && !d.tw_post) {
        const int t = p * k1o;
        if (t) v[n1] = v[n1] * twid<R>(full_tab<R>(d), t, sign);
      }
    }
    Dft<R, A>::run(v, sign, line_tab<R>(d), L);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      cx<R> w = v[k1];
      if (k1 && n2) w = w * twid<R>(line_tab<R>(d), n2 * k1, sign);
      sm[slot(b, k1, n2)] = w;
    }
  }
  __syncthreads();
  // phase 2: DFT over n2, write X[k1 + A k2]
  for (int it = threadIdx.x; it < nl * A; it += blockDim.x) {
    int b, k1;
    if (contig) { k1 = it % A; b = it / A; } else { b = it % nl; k1 = it / nl; }
    if (b >= nact) continue;
    cx<R> u[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) u[n2] = sm[slot(b, k1, n2)];
    Dft<R, B>::run(u, sign, line_tab<R>(d), L);
    const int k1o = tw4 ? (int)((contig ? o + b : o) % d.tw_L1) : 0;
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) {
      const int q = k1 + A * k2;
      cx<R> w = u[k2];
      if (tw4 && d.tw_post) {
        const int t = q * k1o;  // q < L2, k1o < L1
        if (t) w = w * twid<R>(full_tab<R>(d), t, sign);
      }
      const long long addr = contig ? base + (long long)b * L + q : base + (long long)q * d.S + b;
      arr[addr] = w;
    }
  }
}

// (A, B) pairs with a compiled two-level kernel
constexpr int kFastPairs[][2] = {{8, 8}, {4, 8}, {8, 4}, {4, 4}, {2, 8}, {8, 2}, {2, 4}, {4, 2}, {2, 2},
                                 {3, 8}, {8, 3}, {3, 4}, {4, 3}, {3, 3}, {2, 3}, {3, 2}, {5, 5}, {4, 5},
                                 {5, 4}, {2, 5}, {5, 2}, {3, 5}, {5, 3}, {5, 8}, {8, 5}};

bool fast_pair(int L, int* a, int* b) {
  int best = -1;
  for (int i = 0; i < (int)(sizeof(kFastPairs) / sizeof(kFastPairs[0])); ++i) {
    const int x = kFastPairs[i][0], y = kFastPairs[i][1];
    if (x * y != L) continue;
    if (best < 0 || std::abs(x - y) < std::abs(kFastPairs[best][0] - kFastPairs[best][1])) best = i;
  }
  if (best < 0) return false;
  *a = kFastPairs[best][0];
  *b = kFastPairs[best][1];
  return true;
}

// ------------------------------------------------ TMA-staged strided pass
// A strided pass of the two-level kernel whose tiles move by TMA.  The pass's
// data is a 2-D tensor: dim0 = the S contiguous elements of a row (counted in
// 8-byte words), dim1 = the rows (stride S elements) of all arrays of the
// launch.  A tile is the box of kTmaLines adjacent lines x L points; it lands
// in shared memory as [point][line], so the phase-1 reads and the phase-2
// writes (line fastest across threads) are conflict-free, and the tile goes
// back by a TMA store from the same buffer.  A CTA is persistent over tiles
// and double-buffers them: the load of tile i + 2 is issued as soon as the
// store of tile i has read its buffer.  Every wait on an mbarrier is bounded
// (kTmaWaitCycles); a CTA that gives up sets the mapped host flag, waits
// (bounded) for its own loads still in flight and returns, and the host
// raises at its next synchronization.
constexpr int kTmaLines = 32;
constexpr long long kTmaWaitCycles = 4000000000LL;  // about 2 s at 2 GHz

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; false if the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kTmaWaitCycles) return false;
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
               ::"l"(map), "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}

template <typename R, int A, int B>
__global__ void __launch_bounds__(256) fft2_tma_kernel(const __grid_constant__ CUtensorMap map, PassDesc d,
                                                       long long nsb, long long ntiles, long long rows_per_array,
                                                       int sign, volatile int* err) {
  constexpr int L = A * B, NL = kTmaLines;
  constexpr int W = (int)(sizeof(cx<R>) / 8);  // 8-byte words per element
  constexpr unsigned kTileBytes = (unsigned)(L * NL * sizeof(cx<R>));
  extern __shared__ __align__(128) unsigned char smem_raw[];
  cx<R>* bufs = reinterpret_cast<cx<R>*>(smem_raw);  // [2][L][NL]
  cx<R>* xch = bufs + 2 * L * NL;                     // [A][B][NL]
  uint64_t* bar = reinterpret_cast<uint64_t*>(xch + L * NL);
  const long long per_array = d.O * nsb;
  auto coord = [&](long long t, int& x, int& y, long long& o) {
    const long long a = t / per_array, rem = t - a * per_array;
    o = rem / nsb;
    x = (int)((rem - o * nsb) * NL * W);
    y = (int)(a * rows_per_array + o * L);
  };
  const long long step = gridDim.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0]);
    mbar_init(&bar[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int k = 0; k < 2; ++k) {
      const long long t = blockIdx.x + k * step;
      if (t < ntiles) {
        int x, y;
        long long o;
        coord(t, x, y, o);
        mbar_expect_tx(&bar[k], kTileBytes);
        tma_load_2d(bufs + k * L * NL, &map, x, y, &bar[k]);
      }
    }
  }
  __syncthreads();
  const bool tw4 = d.tw_L1 > 0;
  unsigned parity[2] = {0u, 0u};
  bool bad = false;
  int it = 0;
  for (long long t = blockIdx.x; t < ntiles; t += step, ++it) {
    const int cur = it & 1;
    cx<R>* buf = bufs + cur * L * NL;
    bool ok = mbar_wait(&bar[cur], parity[cur]);
    if (__syncthreads_or(!ok)) {
      bad = true;
      break;
    }
    parity[cur] ^= 1u;
    int x, y;
    long long o;
    coord(t, x, y, o);
    const int k1o = tw4 ? (int)(o % d.tw_L1) : 0;
    // phase 1: A points per (line, n2), DFT over n1, inner twiddle
    for (int item = threadIdx.x; item < NL * B; item += blockDim.x) {
      const int b = item % NL, n2 = item / NL;
      cx<R> v[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) {
        const int p = B * n1 + n2;
        v[n1] = buf[p * NL + b];
        if (tw4 && !d.tw_post) {
          const int tt = p * k1o;
          if (tt) v[n1] = v[n1] * twid<R>(full_tab<R>(d), tt, sign);
        }
      }
      Dft<R, A>::run(v, sign, line_tab<R>(d), L);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) {
        cx<R> w = v[k1];
        if (k1 && n2) w = w * twid<R>(line_tab<R>(d), n2 * k1, sign);
        xch[(k1 * B + n2) * NL + b] = w;
      }
    }
    __syncthreads();
    // phase 2: DFT over n2, X[k1 + A k2] back into the tile buffer
    for (int item = threadIdx.x; item < NL * A; item += blockDim.x) {
      const int b = item % NL, k1 = item / NL;
      cx<R> u[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) u[n2] = xch[(k1 * B + n2) * NL + b];
      Dft<R, B>::run(u, sign, line_tab<R>(d), L);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) {
        const int q = k1 + A * k2;
        cx<R> w = u[k2];
        if (tw4 && d.tw_post) {
          const int tt = q * k1o;
          if (tt) w = w * twid<R>(full_tab<R>(d), tt, sign);
        }
        buf[q * NL + b] = w;
      }
    }
    // the generic-proxy writes of the tile become visible to the TMA store
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store_2d(&map, x, y, buf);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      const long long tn = t + 2 * step;
      if (tn < ntiles) {
        // the buffer is reloaded only after the store has read it
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        int xn, yn;
        long long on;
        coord(tn, xn, yn, on);
        mbar_expect_tx(&bar[cur], kTileBytes);
        tma_load_2d(buf, &map, xn, yn, &bar[cur]);
      }
    }
  }
  if (threadIdx.x == 0) {
    if (bad) {
      *err = 1;
      // the loads this CTA issued and has not consumed: tiles it + 0 and
      // it + 1 of the loop, each bounded
      for (int k = 0; k < 2; ++k) {
        const long long t = blockIdx.x + (long long)(it + k) * step;
        if (t < ntiles) mbar_wait(&bar[(it + k) & 1], parity[(it + k) & 1]);
      }
    }
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
}

// x and y of each (x, y) plane of side L = A B in one pass (nx == ny == L):
// the plane is read once into shared memory, both axes are transformed there
// with the two-level register scheme of fft2_kernel (radix A, twiddle, radix
// B; natural order out), and the plane is written once.  Rows are padded to
// L + 1 and every phase runs the line index fastest across threads, so the
// row-wise (stride L + 1) and column-wise (stride 1) accesses are free of
// bank conflicts for 8- and 16-byte elements.  Each thread keeps its phase
// inputs in registers across the barriers, so the exchange of a phase
// reuses the plane buffer: L (L + 1) elements of shared memory in all.
template <typename R, int A, int B>
__global__ void __launch_bounds__(256) fft_xy_kernel(cx<R>* data, long long P, PassDesc d, int sign) {
  constexpr int L = A * B, RS = L + 1;
  constexpr int NI1 = (L * B + 255) / 256, NI2 = (L * A + 255) / 256;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<R>* sm = reinterpret_cast<cx<R>*>(smem_raw);
  cx<R>* g = data + (long long)blockIdx.y * P + (long long)blockIdx.x * (L * L);
  const cx<R>* tab = line_tab<R>(d);
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) sm[(e / L) * RS + (e % L)] = g[e];
  __syncthreads();
#pragma unroll 1
  for (int axis = 0; axis < 2; ++axis) {
    // axis 0: line l = row y, position p = x; axis 1: line l = column x, p = y
    const int es = axis == 0 ? 1 : RS, ls = axis == 0 ? RS : 1;
    cx<R> v[NI1][A];
#pragma unroll
    for (int i = 0; i < NI1; ++i) {
      const int it = threadIdx.x + 256 * i;
      if (it < L * B) {
        const int l = it % L, n2 = it / L;
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) v[i][n1] = sm[l * ls + (B * n1 + n2) * es];
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NI1; ++i) {
      const int it = threadIdx.x + 256 * i;
      if (it < L * B) {
        const int l = it % L, n2 = it / L;
        Dft<R, A>::run(v[i], sign, tab, L);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) {
          cx<R> w = v[i][k1];
          if (k1 && n2) w = w * twid<R>(tab, n2 * k1, sign);
          sm[(k1 * B + n2) * L + l] = w;
        }
      }
    }
    __syncthreads();
    cx<R> u[NI2][B];
#pragma unroll
    for (int j = 0; j < NI2; ++j) {
      const int it = threadIdx.x + 256 * j;
      if (it < L * A) {
        const int l = it % L, k1 = it / L;
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) u[j][n2] = sm[(k1 * B + n2) * L + l];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NI2; ++j) {
      const int it = threadIdx.x + 256 * j;
      if (it < L * A) {
        const int l = it % L, k1 = it / L;
        Dft<R, B>::run(u[j], sign, tab, L);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) sm[l * ls + (k1 + A * k2) * es] = u[j][k2];
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) g[e] = sm[(e / L) * RS + (e % L)];
}

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// the current context's timeout flag of the TMA passes, in mapped pinned
// host memory
int* tma_flag() {
  Context& c = ctx();
  if (!c.tma_flag_h) {
    void* h = nullptr;
    PGB_CUDA(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped));
    *static_cast<volatile int*>(h) = 0;
    void* dptr = nullptr;
    PGB_CUDA(cudaHostGetDevicePointer(&dptr, h, 0));
    c.tma_flag_d = static_cast<int*>(dptr);
    c.tma_flag_h = static_cast<volatile int*>(h);
  }
  return c.tma_flag_d;
}

// TMA-staged strided passes: on for 8-byte elements (c2's FP32 4-D transform
// 0.381 -> 0.360 ms), off for 16-byte ones (1.27 -> 1.29 ms); PYRPA_GB_FFT_TMA
// = 1 / 0 forces them on / off
bool tma_pass_enabled(int elem_bytes) {
  const char* s = std::getenv("PYRPA_GB_FFT_TMA");
  if (s) return std::string(s) == "1";
  return elem_bytes == 8;
}

template <typename R, int A, int B>
void launch_tma_ab(const CUtensorMap& map, const PassDesc& d, long long nsb, long long ntiles, long long rows,
                   cudaStream_t s, int sign) {
  constexpr int L = A * B;
  const size_t smem = (size_t)3 * L * kTmaLines * sizeof(cx<R>) + 2 * sizeof(uint64_t);
  static const int per_sm = [&] {
    int n = 0;
    PGB_CUDA(cudaFuncSetAttribute(fft2_tma_kernel<R, A, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fft2_tma_kernel<R, A, B>, 256, smem));
    return std::max(1, n);
  }();
  const long long grid = std::max(1LL, std::min<long long>(ntiles, (long long)ctx().num_sms * per_sm));
  fft2_tma_kernel<R, A, B><<<(unsigned)grid, 256, smem, s>>>(map, d, nsb, ntiles, rows, sign, tma_flag());
}

template <typename R>
void launch_tma(const PassDesc& d, long long nbb, cudaStream_t s, cx<R>* data, long long P, int sign) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
  PGB_CHECK(enc != nullptr, "cuTensorMapEncodeTiled is not available from the driver");
  constexpr int W = (int)(sizeof(cx<R>) / 8);
  const long long rows = P / d.S;  // P = O L S: rows of S elements per array
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)(d.S * W), (cuuint64_t)(rows * nbb)};
  const cuuint64_t strides[1] = {(cuuint64_t)(d.S * sizeof(cx<R>))};
  const cuuint32_t box[2] = {(cuuint32_t)(kTmaLines * W), (cuuint32_t)d.L};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, static_cast<void*>(data), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  PGB_CHECK(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed for an FFT pass (code " + std::to_string((int)r) + ")");
  const long long nsb = d.S / kTmaLines, ntiles = nbb * d.O * nsb;
#define PGB_TMA(A_, B_)                                                 \
  if (d.fa == A_ && d.fb == B_) {                                       \
    launch_tma_ab<R, A_, B_>(map, d, nsb, ntiles, rows, s, sign);        \
    return;                                                             \
  }
  PGB_TMA(8, 8) PGB_TMA(4, 8) PGB_TMA(8, 4) PGB_TMA(4, 4) PGB_TMA(2, 8) PGB_TMA(8, 2) PGB_TMA(3, 8) PGB_TMA(8, 3)
  PGB_TMA(2, 4) PGB_TMA(4, 2) PGB_TMA(3, 4) PGB_TMA(4, 3)
#undef PGB_TMA
  throw Error("no TMA FFT kernel for this line length");
}

bool tma_pair(int a, int b) {
  const int ok[][2] = {{8, 8}, {4, 8}, {8, 4}, {4, 4}, {2, 8}, {8, 2}, {3, 8}, {8, 3}, {2, 4}, {4, 2}, {3, 4}, {4, 3}};
  for (const auto& x : ok)
    if (x[0] == a && x[1] == b) return true;
  return false;
}

template <typename R>
void launch_xy(const PassDesc& d, dim3 grid, cudaStream_t s, cx<R>* data, long long P, int sign) {
  const size_t smem = (size_t)d.L * (d.L + 1) * sizeof(cx<R>);
#define PGB_XY(A_, B_)                                                                              \
  if (d.fa == A_ && d.fb == B_) {                                                                   \
    PGB_SMEM_LIMIT_ONCE((fft_xy_kernel<R, A_, B_>), smem);                                          \
    fft_xy_kernel<R, A_, B_><<<grid, 256, smem, s>>>(data, P, d, sign);                             \
    return;                                                                                         \
  }
  PGB_XY(8, 8) PGB_XY(4, 8) PGB_XY(8, 4) PGB_XY(4, 4) PGB_XY(3, 8) PGB_XY(8, 3) PGB_XY(2, 8) PGB_XY(8, 2)
  PGB_XY(3, 4) PGB_XY(4, 3) PGB_XY(2, 4) PGB_XY(4, 2)
#undef PGB_XY
  throw Error("no x-y plane FFT kernel for this side");
}

// the sides the x-y plane pass takes (square planes; 16-byte elements of a
// 64 x 64 plane fill 66.6 KB of shared memory)
bool xy_side(int L, int* a, int* b) {
  if (!fast_pair(L, a, b)) return false;
  const int ok[][2] = {{8, 8}, {4, 8}, {8, 4}, {4, 4}, {3, 8}, {8, 3}, {2, 8}, {8, 2}, {3, 4}, {4, 3}, {2, 4}, {4, 2}};
  for (const auto& x : ok)
    if (x[0] == *a && x[1] == *b) return true;
  return false;
}

// the x-y plane pass is on unless PYRPA_GB_FFT_XY=0
bool xy_pass_enabled() {
  const char* s = std::getenv("PYRPA_GB_FFT_XY");
  return !(s && std::string(s) == "0");
}

template <typename R>
void launch_fast(const PassDesc& d, dim3 grid, size_t smem, cudaStream_t s, cx<R>* data, long long P, int sign) {
#define PGB_FAST(A_, B_)                                                                    \
  if (d.fa == A_ && d.fb == B_) {                                                           \
    fft2_kernel<R, A_, B_><<<grid, 256, smem, s>>>(data, P, d, sign);                       \
    return;                                                                                 \
  }
  PGB_FAST(8, 8) PGB_FAST(4, 8) PGB_FAST(8, 4) PGB_FAST(4, 4) PGB_FAST(2, 8) PGB_FAST(8, 2)
  PGB_FAST(2, 4) PGB_FAST(4, 2) PGB_FAST(2, 2) PGB_FAST(3, 8) PGB_FAST(8, 3) PGB_FAST(3, 4)
  PGB_FAST(4, 3) PGB_FAST(3, 3) PGB_FAST(2, 3) PGB_FAST(3, 2) PGB_FAST(5, 5) PGB_FAST(4, 5)
  PGB_FAST(5, 4) PGB_FAST(2, 5) PGB_FAST(5, 2) PGB_FAST(3, 5) PGB_FAST(5, 3) PGB_FAST(5, 8)
  PGB_FAST(8, 5)
#undef PGB_FAST
  throw Error("no two-level FFT kernel for this line length");
}

std::mutex g_mu;
std::map<int, double2*> g_tables;
std::map<int, float2*> g_tables_f;
std::map<int, cdf*> g_tables_d;

struct PassEvent {
  cudaEvent_t a, b;
  double bytes;
};
bool g_prof = false;
std::vector<PassEvent> g_prof_ev;
std::vector<cudaEvent_t> g_ev_pool;
cudaEvent_t take_event() {
  if (!g_ev_pool.empty()) {
    cudaEvent_t e = g_ev_pool.back();
    g_ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  PGB_CUDA(cudaEventCreate(&e));
  return e;
}

const double2* twiddle_table(int L) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(L);
  if (it != g_tables.end()) return it->second;
  std::vector<double2> h(L);
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (int t = 0; t < L; ++t) {
    // reduce to the first octant-free form: exact values at quarter turns
    long long q = (long long)t * 4;
    if (q % L == 0) {
      int quarter = (int)((q / L) % 4);
      const double c[4] = {1.0, 0.0, -1.0, 0.0}, s[4] = {0.0, 1.0, 0.0, -1.0};
      h[t] = make_double2(c[quarter], -s[quarter]);
    } else {
      long double a = twopi * (long double)t / (long double)L;
      h[t] = make_double2((double)cosl(a), (double)(-sinl(a)));
    }
  }
  double2* d = nullptr;
  PGB_CUDA(cudaMalloc(&d, sizeof(double2) * L));
  PGB_CUDA(cudaMemcpy(d, h.data(), sizeof(double2) * L, cudaMemcpyHostToDevice));
  g_tables[L] = d;
  std::vector<float2> hf(L);
  for (int t = 0; t < L; ++t) hf[t] = make_float2((float)h[t].x, (float)h[t].y);
  float2* df = nullptr;
  PGB_CUDA(cudaMalloc(&df, sizeof(float2) * L));
  PGB_CUDA(cudaMemcpy(df, hf.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
  g_tables_f[L] = df;
  // double-float copy: hi = float(root), lo = float(root - hi) from the
  // extended-precision value
  std::vector<cdf> hd(L);
  for (int t = 0; t < L; ++t) {
    long double c = h[t].x, s = h[t].y;
    long long q = (long long)t * 4;
    if (q % L != 0) {
      const long double a = twopi * (long double)t / (long double)L;
      c = cosl(a);
      s = -sinl(a);
    }
    const float ch = (float)c, sh = (float)s;
    hd[t] = mkc(dfl(ch, (float)(c - (long double)ch)), dfl(sh, (float)(s - (long double)sh)));
  }
  cdf* dd = nullptr;
  PGB_CUDA(cudaMalloc(&dd, sizeof(cdf) * L));
  PGB_CUDA(cudaMemcpy(dd, hd.data(), sizeof(cdf) * L, cudaMemcpyHostToDevice));
  // a copy from pageable memory may still be in flight when cudaMemcpy
  // returns, and the tables are read from every thread's stream
  PGB_CUDA(cudaDeviceSynchronize());
  g_tables_d[L] = dd;
  return d;
}

const float2* twiddle_table_f(int L) {
  twiddle_table(L);
  std::lock_guard<std::mutex> lk(g_mu);
  return g_tables_f[L];
}

const cdf* twiddle_table_d(int L) {
  twiddle_table(L);
  std::lock_guard<std::mutex> lk(g_mu);
  return g_tables_d[L];
}

bool factor_line(int L, int* radix, int* nst) {
  int n = L, k = 0;
  const int pref[] = {8, 4, 2, 3, 5, 7, 11, 13};
  for (int r : pref) {
    while (n % r == 0 && n > 1) {
      if (k >= kMaxStages) return false;
      radix[k++] = r;
      n /= r;
    }
  }
  *nst = k;
  return n == 1;
}

PassDesc make_pass(int L, long long S, long long O, int elem_bytes, int lines = 0) {
  PassDesc d{};
  d.L = L;
  d.S = S;
  d.O = O;
  if (fast_pair(L, &d.fa, &d.fb)) {
    long long nl = std::max(1, 2048 / L);
    nl = std::min(nl, 64LL);
    if (lines > 0) nl = lines;
    nl = (S == 1) ? std::min(nl, O) : std::min(nl, S);
    d.B = (int)std::max(1LL, nl);
    d.tw_line = twiddle_table(L);
    d.tw_line_f = twiddle_table_f(L);
    d.tw_line_d = twiddle_table_d(L);
    d.nst = 0;
    return d;
  }
  d.fa = d.fb = 0;
  PGB_CHECK(factor_line(L, d.radix, &d.nst),
            "FFT length " + std::to_string(L) + " has a prime factor above 13 (unsupported)");
  long long B = std::max(1LL, 32768LL / ((long long)L * elem_bytes));
  B = std::min(B, 64LL);
  if (lines > 0) B = lines;
  if (S == 1) B = std::min(B, O);
  else B = std::min(B, S);
  d.B = (int)std::max(1LL, B);
  d.tw_line = twiddle_table(L);
  d.tw_line_f = twiddle_table_f(L);
  d.tw_line_d = twiddle_table_d(L);
  return d;
}

constexpr int kMaxPlaneSide = 64;  // two padded 64 x 65 planes of 16-byte elements fit in 227 KB

// PYRPA_GB_FFT_LONG=1 transforms four-step axes of length L1 L2 (L1, L2 in
// {16, 64}) in one long pass
bool long_pass_enabled() {
  const char* s = std::getenv("PYRPA_GB_FFT_LONG");
  return s && std::string(s) == "1";
}

bool long_split(int n, int* l1, int* l2) {
  const int sp[4][2] = {{64, 64}, {16, 64}, {64, 16}, {16, 16}};
  for (const auto& x : sp)
    if (x[0] * x[1] == n) {
      *l1 = x[0];
      *l2 = x[1];
      return true;
    }
  return false;
}

// PYRPA_GB_FFT_PLANE=1 transforms x and y in one plane pass
bool plane_pass_enabled() {
  const char* s = std::getenv("PYRPA_GB_FFT_PLANE");
  return s && std::string(s) == "1";
}

int split_length(int n) {
  // L1 * L2 = n with both <= kMaxLine, L1 as close to sqrt(n) as possible
  int best = -1;
  for (int a = 2; a <= kMaxLine; ++a) {
    if (n % a) continue;
    int b = n / a;
    if (b > kMaxLine) continue;
    if (best < 0 || std::abs(a - b) < std::abs(best - n / best)) best = a;
  }
  PGB_CHECK(best > 0, "FFT axis length " + std::to_string(n) + " cannot be split into passes");
  return best;
}

}  // namespace

FFT4D::FFT4D(int nx, int ny, int nz, int nt, int elem_bytes, const PlanTune* tune) {
  dims_[0] = nx;
  dims_[1] = ny;
  dims_[2] = nz;
  dims_[3] = nt;
  P_ = (long long)nx * ny * nz * nt;
  std::vector<int> tables;
  long long S = 1;
  for (int a = 0; a < 4; ++a) {
    const int n = dims_[a];
    const long long O = P_ / (S * n);
    AxisMap& m = maps_[a];
    m.n = n;
    m.pos.resize(n);
    m.logical.resize(n);
    m.rev.resize(n);
    int fa = 0, fb = 0, L1s = 0;
    const AxisTune tn = tune ? tune->ax[a] : AxisTune{};
    const bool direct_fast = fast_pair(n, &fa, &fb);
    int ta, tb, lp1 = 0, lp2 = 0;
    if (n > 64 && !direct_fast && tn.L1 > 0 && n % tn.L1 == 0 && n / tn.L1 <= 64 && fast_pair(tn.L1, &ta, &tb) &&
        fast_pair(n / tn.L1, &ta, &tb)) {
      L1s = tn.L1;
    } else if (n > 64 && !direct_fast) {
      // four-step split into two lengths that both have a two-level kernel
      int best = -1;
      for (int a1 = 2; a1 <= 64; ++a1) {
        if (n % a1 || n / a1 > 64) continue;
        int x, y, z, w;
        if (!fast_pair(a1, &x, &y) || !fast_pair(n / a1, &z, &w)) continue;
        if (best < 0 || std::abs(a1 - n / a1) < std::abs(best - n / best)) best = a1;
      }
      L1s = best > 0 ? best : 0;
    }
    if (n > 1 && L1s == 0 && n <= kMaxLine) {
      PassDesc p = make_pass(n, S, O, elem_bytes, tn.lines);
      fwd_.push_back(p);
      bwd_.push_back(p);
      if (a < 3) {
        fwd_space_.push_back(p);
        bwd_space_.push_back(p);
      }
      for (int k = 0; k < n; ++k) m.pos[k] = k;
    } else if (n > 1 && long_pass_enabled() && long_split(n, &lp1, &lp2)) {
      // the whole axis in one long pass, digit-transposed like the four-step split
      const int L1 = lp1, L2 = lp2;
      PassDesc lp{};
      lp.lp = 1;
      lp.L = n;
      lp.lp_L1 = L1;
      lp.lp_L2 = L2;
      lp.S = S;
      lp.O = O;
      const long long fit = (long long)(kLongSmem / ((size_t)L1 * (L2 + 1) * elem_bytes));
      // a power of two, so that each CTA's runs start on 32-byte sectors
      long long nb = 1;
      while (nb * 2 <= std::min({32LL, fit, S})) nb *= 2;
      lp.B = (int)nb;
      lp.tw_line = twiddle_table(L1);
      lp.tw_line_f = twiddle_table_f(L1);
      lp.tw_line_d = twiddle_table_d(L1);
      lp.tw_line_y = twiddle_table(L2);
      lp.tw_line_y_f = twiddle_table_f(L2);
      lp.tw_line_y_d = twiddle_table_d(L2);
      lp.tw_full = twiddle_table(n);
      lp.tw_full_f = twiddle_table_f(n);
      lp.tw_full_d = twiddle_table_d(n);
      fwd_.push_back(lp);
      bwd_.push_back(lp);
      if (a < 3) {
        fwd_space_.push_back(lp);
        bwd_space_.push_back(lp);
      }
      for (int k = 0; k < n; ++k) m.pos[k] = (k / L1) + L2 * (k % L1);
    } else if (n > 1) {
      const int L1 = L1s ? L1s : split_length(n), L2 = n / L1;
      PassDesc pb = make_pass(L1, S * L2, O, elem_bytes, tn.lines);
      PassDesc pa = make_pass(L2, S, O * L1, elem_bytes, tn.lines);
      pa.tw_L1 = L1;
      pa.tw_Lfull = n;
      pa.tw_full = twiddle_table(n);
      pa.tw_full_f = twiddle_table_f(n);
      pa.tw_full_d = twiddle_table_d(n);
      PassDesc pa_inv = pa;
      pa_inv.tw_post = 1;
      fwd_.push_back(pb);
      fwd_.push_back(pa);
      bwd_.push_back(pa_inv);
      bwd_.push_back(pb);
      if (a < 3) {
        fwd_space_.push_back(pb);
        fwd_space_.push_back(pa);
        bwd_space_.push_back(pa_inv);
        bwd_space_.push_back(pb);
      }
      for (int k = 0; k < n; ++k) m.pos[k] = (k / L1) + L2 * (k % L1);
    } else {
      m.pos[0] = 0;
    }
    for (int k = 0; k < n; ++k) m.logical[m.pos[k]] = k;
    for (int p = 0; p < n; ++p) m.rev[p] = m.pos[(n - m.logical[p]) % n];
    S *= n;
  }
  // x and y of square planes in one two-level pass (default), else the
  // opt-in Stockham plane pass
  int xa = 0, xb = 0;
  if (xy_pass_enabled() && !plane_pass_enabled() && nx == ny && nx > 1 && xy_side(nx, &xa, &xb)) {
    PassDesc xy = fwd_[0];
    xy.xy = 1;
    xy.L = nx;
    xy.S = 1;
    xy.O = P_ / ((long long)nx * ny);
    xy.B = 1;
    xy.fa = xa;
    xy.fb = xb;
    for (auto* v : {&fwd_, &bwd_, &fwd_space_, &bwd_space_}) {
      v->erase(v->begin(), v->begin() + 2);
      v->insert(v->begin(), xy);
    }
  } else if (plane_pass_enabled() && nx >= 2 && ny >= 2 && nx <= kMaxPlaneSide && ny <= kMaxPlaneSide) {
    PassDesc pl{};
    pl.plane = 1;
    pl.L = nx;
    pl.ny = ny;
    pl.S = 1;
    pl.O = P_ / ((long long)nx * ny);
    pl.B = 1;
    if (factor_line(nx, pl.radix, &pl.nst) && factor_line(ny, pl.radix_y, &pl.nst_y)) {
      pl.tw_line = twiddle_table(nx);
      pl.tw_line_f = twiddle_table_f(nx);
      pl.tw_line_d = twiddle_table_d(nx);
      pl.tw_line_y = twiddle_table(ny);
      pl.tw_line_y_f = twiddle_table_f(ny);
      pl.tw_line_y_d = twiddle_table_d(ny);
      // sides <= 64 are direct passes, so x and y are the first two passes of every list
      for (auto* v : {&fwd_, &bwd_, &fwd_space_, &bwd_space_}) {
        v->erase(v->begin(), v->begin() + 2);
        v->insert(v->begin(), pl);
      }
    }
  }
  // strided two-level passes staged by TMA
  if (tma_pass_enabled(elem_bytes)) {
    for (auto* v : {&fwd_, &bwd_, &fwd_space_, &bwd_space_})
      for (PassDesc& p : *v)
        if (p.fa && !p.xy && !p.plane && !p.lp && p.S > 1 && p.S % kTmaLines == 0 && tma_pair(p.fa, p.fb))
          p.tma = 1;
  }
  // device tables
  std::vector<int> h;
  for (int a = 0; a < 4; ++a) {
    off_pos_[a] = (int)h.size();
    h.insert(h.end(), maps_[a].pos.begin(), maps_[a].pos.end());
    off_rev_[a] = (int)h.size();
    h.insert(h.end(), maps_[a].rev.begin(), maps_[a].rev.end());
    off_log_[a] = (int)h.size();
    h.insert(h.end(), maps_[a].logical.begin(), maps_[a].logical.end());
  }
  PGB_CUDA(cudaMalloc(&d_tables_, sizeof(int) * h.size()));
  PGB_CUDA(cudaMemcpy(d_tables_, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice));
  PGB_CUDA(cudaDeviceSynchronize());  // complete before any thread's stream reads them
}

template <typename R>
void FFT4D::run(const std::vector<PassDesc>& passes, cx<R>* data, int nb, int sign,
                cudaStream_t s) const {
  PGB_SMEM_LIMIT_ONCE(fft_pass_kernel<R>, 96 * 1024);
  for (const PassDesc& d : passes) {
    const long long tiles = (d.plane || d.xy) ? d.O
                            : d.lp ? d.O * ((d.S + d.B - 1) / d.B)
                            : (d.S == 1) ? (d.O + d.B - 1) / d.B : d.O * ((d.S + d.B - 1) / d.B);
    const size_t smem = d.plane ? 2 * (size_t)d.ny * (d.L + 1) * sizeof(cx<R>)
                        : d.lp  ? (size_t)d.B * d.lp_L1 * (d.lp_L2 + 1) * sizeof(cx<R>)
                        : d.fa  ? (size_t)d.B * d.fa * (d.fb + 1) * sizeof(cx<R>)
                                : 2 * (size_t)d.B * d.L * sizeof(cx<R>);
    for (int b0 = 0; b0 < nb; b0 += 65535) {
      const int nbb = std::min(65535, nb - b0);
      dim3 grid((unsigned)tiles, (unsigned)nbb);
      PassEvent pe{};
      if (g_prof) {
        pe.a = take_event();
        pe.b = take_event();
        pe.bytes = 2.0 * (double)nbb * (double)P_ * sizeof(cx<R>);
        PGB_CUDA(cudaEventRecord(pe.a, s));
      }
      if (d.plane) {
        PGB_SMEM_LIMIT_ONCE(fft_plane_kernel<R>, 2 * kMaxPlaneSide * (kMaxPlaneSide + 1) * sizeof(cx<R>));
        fft_plane_kernel<R><<<grid, 256, smem, s>>>(data + (long long)b0 * P_, P_, d, sign);
      }
      else if (d.xy) launch_xy<R>(d, grid, s, data + (long long)b0 * P_, P_, sign);
      else if (d.tma) launch_tma<R>(d, nbb, s, data + (long long)b0 * P_, P_, sign);
      else if (d.lp) launch_long<R>(d, grid, smem, s, data + (long long)b0 * P_, P_, sign);
      else if (d.fa) launch_fast<R>(d, grid, smem, s, data + (long long)b0 * P_, P_, sign);
      else fft_pass_kernel<R><<<grid, 256, smem, s>>>(data + (long long)b0 * P_, P_, d, sign);
      launch_check("fft_pass");
      if (g_prof) {
        PGB_CUDA(cudaEventRecord(pe.b, s));
        g_prof_ev.push_back(pe);
      }
      ctx().kernel_launches++;
    }
  }
}

template <typename R> void FFT4D::forward(cx<R>* data, int nb, cudaStream_t s) const {
  run<R>(fwd_, data, nb, -1, s);
}
template <typename R> void FFT4D::backward(cx<R>* data, int nb, cudaStream_t s) const {
  run<R>(bwd_, data, nb, +1, s);
}
template <typename R> void FFT4D::forward_space(cx<R>* data, int nb, cudaStream_t s) const {
  run<R>(fwd_space_, data, nb, -1, s);
}
template <typename R> void FFT4D::backward_space(cx<R>* data, int nb, cudaStream_t s) const {
  run<R>(bwd_space_, data, nb, +1, s);
}

template void FFT4D::forward<float>(float2*, int, cudaStream_t) const;
template void FFT4D::forward<double>(double2*, int, cudaStream_t) const;
template void FFT4D::backward<float>(float2*, int, cudaStream_t) const;
template void FFT4D::backward<double>(double2*, int, cudaStream_t) const;
template void FFT4D::forward_space<float>(float2*, int, cudaStream_t) const;
template void FFT4D::forward_space<double>(double2*, int, cudaStream_t) const;
template void FFT4D::backward_space<float>(float2*, int, cudaStream_t) const;
template void FFT4D::backward_space<double>(double2*, int, cudaStream_t) const;
template void FFT4D::forward<dfl>(cdf*, int, cudaStream_t) const;
template void FFT4D::backward<dfl>(cdf*, int, cudaStream_t) const;
template void FFT4D::forward_space<dfl>(cdf*, int, cudaStream_t) const;
template void FFT4D::backward_space<dfl>(cdf*, int, cudaStream_t) const;

void fft_profile_enable(bool on) { g_prof = on; }

void fft_raise_pending() {
  Context& c = ctx();
  if (c.tma_flag_h && *c.tma_flag_h) {
    *c.tma_flag_h = 0;
    throw Error("an FFT pass gave up waiting for its TMA copies (bounded wait ran out)");
  }
}

void fft_profile_collect(double* launches, double* ms, double* bytes) {
  double n = 0, t = 0, b = 0;
  for (auto& e : g_prof_ev) {
    PGB_CUDA(cudaEventSynchronize(e.b));
    float x = 0;
    PGB_CUDA(cudaEventElapsedTime(&x, e.a, e.b));
    n += 1;
    t += x;
    b += e.bytes;
    g_ev_pool.push_back(e.a);
    g_ev_pool.push_back(e.b);
  }
  g_prof_ev.clear();
  *launches = n;
  *ms = t;
  *bytes = b;
}

void FFT4D::release_tables() {
  if (d_tables_) cudaFree(d_tables_);
  d_tables_ = nullptr;
}

namespace {

// shared memory of one pass of length L with `lines` lines per CTA, and
// whether it fits that kernel's launch (48 KB for the two-level kernel,
// 96 KB for the Stockham kernel, the limits the plan's launches use)
bool pass_fits(int L, int lines, int elem_bytes) {
  int a, b;
  if (fast_pair(L, &a, &b)) return (long long)lines * a * (b + 1) * elem_bytes <= 48 * 1024;
  return 2LL * lines * L * elem_bytes <= 96 * 1024;
}

bool tune_enabled() {
  const char* s = std::getenv("PYRPA_GB_FFT_TUNE");
  return s && std::string(s) == "1";
}

// the fastest of each axis's candidates, one axis after another, timed as
// whole forward transforms of one scratch array (min of 3 after a warm-up)
template <typename R>
PlanTune tune_plan(int nx, int ny, int nz, int nt) {
  const int dims[4] = {nx, ny, nz, nt};
  const long long P = (long long)nx * ny * nz * nt;
  cudaStream_t st = ctx().stream;
  DBuf<cx<R>> x(P);
  x.zero();
  cudaEvent_t e0, e1;
  PGB_CUDA(cudaEventCreate(&e0));
  PGB_CUDA(cudaEventCreate(&e1));
  PlanTune best{};
  for (int a = 0; a < 4; ++a) {
    const std::vector<AxisTune> cands = fft_axis_candidates(dims[a], (int)sizeof(cx<R>));
    if (cands.size() < 2) continue;
    float best_ms = 1e30f;
    AxisTune pick = best.ax[a];
    for (const AxisTune& c : cands) {
      PlanTune trial = best;
      trial.ax[a] = c;
      FFT4D f(nx, ny, nz, nt, (int)sizeof(cx<R>), &trial);
      float ms = 1e30f;
      try {
        f.forward<R>(x.p, 1, st);
        for (int rep = 0; rep < 3; ++rep) {
          PGB_CUDA(cudaEventRecord(e0, st));
          f.forward<R>(x.p, 1, st);
          PGB_CUDA(cudaEventRecord(e1, st));
          PGB_CUDA(cudaEventSynchronize(e1));
          float t = 0;
          PGB_CUDA(cudaEventElapsedTime(&t, e0, e1));
          ms = std::min(ms, t);
        }
      } catch (const Error&) {
        ms = 1e30f;  // a candidate that does not launch is skipped
      }
      f.release_tables();
      if (ms < best_ms) {
        best_ms = ms;
        pick = c;
      }
    }
    best.ax[a] = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

std::vector<AxisTune> fft_axis_candidates(int n, int elem_bytes) {
  std::vector<AxisTune> out;
  if (n <= 1) return out;
  out.push_back(AxisTune{});
  int a, b;
  std::vector<int> splits;
  if (n > 64 && !fast_pair(n, &a, &b)) {
    for (int l1 = 2; l1 <= 64; ++l1)
      if (n % l1 == 0 && n / l1 <= 64 && fast_pair(l1, &a, &b) && fast_pair(n / l1, &a, &b)) splits.push_back(l1);
  } else if (n <= kMaxLine) {
    splits.push_back(0);
  }
  const int lines[] = {8, 16, 32, 64};
  for (int l1 : splits)
    for (int ln : lines) {
      const bool fits = l1 ? (pass_fits(l1, ln, elem_bytes) && pass_fits(n / l1, ln, elem_bytes))
                           : pass_fits(n, ln, elem_bytes);
      if (fits) out.push_back(AxisTune{l1, ln});
    }
  return out;
}

const FFT4D& fft_plan(int nx, int ny, int nz, int nt, int elem_bytes) {
  static std::map<std::tuple<int, int, int, int, int>, FFT4D*> plans;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(nx, ny, nz, nt, elem_bytes);
  auto it = plans.find(key);
  if (it != plans.end()) return *it->second;
  FFT4D* p = nullptr;
  if (tune_enabled() && (elem_bytes == 8 || elem_bytes == 16)) {
    const PlanTune t = elem_bytes == 8 ? tune_plan<float>(nx, ny, nz, nt) : tune_plan<double>(nx, ny, nz, nt);
    p = new FFT4D(nx, ny, nz, nt, elem_bytes, &t);
    log("[FFT] tuned %dx%dx%dx%d (%d-byte): (L1, lines) = (%d,%d) (%d,%d) (%d,%d) (%d,%d)\n", nx, ny, nz, nt,
        elem_bytes, t.ax[0].L1, t.ax[0].lines, t.ax[1].L1, t.ax[1].lines, t.ax[2].L1, t.ax[2].lines, t.ax[3].L1,
        t.ax[3].lines);
  } else {
    p = new FFT4D(nx, ny, nz, nt, elem_bytes);
  }
  plans[key] = p;
  return *p;
}

}  // namespace pgb
