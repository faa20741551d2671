// Learned warm start: features, network forward/backward, Adam, and the
// correction of the seed Sigma.  Declarations and the row/parameter layout:
// lws.cuh.
#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <random>
#include <vector>

#include "lws.cuh"

namespace pgb {
namespace {

constexpr double kPiL = 3.141592653589793238462643383279;
constexpr int kMaxNo = 8;
constexpr int kThr = 256;
constexpr long long kBatchRows = 65536;  // rows per pass over the training set

inline void launched(const char* what) {
  launch_check(what);
  ctx().kernel_launches++;
}

inline unsigned blocks_for(long long n, int threads, long long cap) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// sigma(k, n, a, b), Fortran order with k fastest
__host__ __device__ __forceinline__ long long sidx(long long k, long long n, long long a, long long b, long long Nk,
                                                   long long Nw, long long No) {
  return k + Nk * (n + Nw * (a + No * b));
}

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ double2 zcmul(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ double2 zmulc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ------------------------------------------------------------- features --
// One thread per (k, n) pair: the band-basis matrices U^dagger S U of the
// seed at (k, n) and at (k, 0), and of (fine - seed) at (k, n) when the fine
// Sigma is given, then No^2 rows of 16 features (bf16) and 2 targets.
// Pairs come from kn [P][2] or, when kn is null, are p0 + p = k + Nk * n.
__global__ void k_lws_features(__nv_bfloat16* __restrict__ X, float* __restrict__ T, const double2* __restrict__ ss,
                               const double2* __restrict__ sf, const double2* __restrict__ U,
                               const double* __restrict__ eig, const long long* __restrict__ kn, long long p0,
                               long long P, int Nk, int Nw, int Nw_c, int No, LwsDesc d) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
       p += (long long)gridDim.x * blockDim.x) {
    long long k, n;
    if (kn) {
      k = kn[2 * p];
      n = kn[2 * p + 1];
    } else {
      k = (p0 + p) % Nk;
      n = (p0 + p) / Nk;
    }
    const double2* Uk = U + (long long)No * No * k;  // uni(a, m, k) at a + No * m
    const double* ek = eig + (long long)No * k;      // eig(m, k) at m + No * k
    const double wn = (2.0 * n + 1.0) * kPiL * d.T;
    const double wc = (2.0 * Nw_c - 1.0) * kPiL * d.T;
    for (int j = 0; j < No; ++j) {
      double2 t[kMaxNo], t0[kMaxNo], td[kMaxNo];
      for (int a = 0; a < No; ++a) {
        double2 acc = make_double2(0, 0), acc0 = acc, accd = acc;
        for (int b = 0; b < No; ++b) {
          const double2 u = Uk[b + No * j];
          const double2 s = ss[sidx(k, n, a, b, Nk, Nw, No)];
          acc = zadd(acc, zmul(s, u));
          acc0 = zadd(acc0, zmul(ss[sidx(k, 0, a, b, Nk, Nw, No)], u));
          if (sf) accd = zadd(accd, zmul(zsub(sf[sidx(k, n, a, b, Nk, Nw, No)], s), u));
        }
        t[a] = acc;
        t0[a] = acc0;
        td[a] = accd;
      }
      for (int i = 0; i < No; ++i) {
        double2 s = make_double2(0, 0), s0 = s, sd = s;
        for (int a = 0; a < No; ++a) {
          const double2 u = Uk[a + No * i];
          s = zadd(s, zcmul(u, t[a]));
          s0 = zadd(s0, zcmul(u, t0[a]));
          sd = zadd(sd, zcmul(u, td[a]));
        }
        double f[kLwsNF];
        f[0] = s.x / d.s_scale;
        f[1] = s.y / d.s_scale;
        f[2] = (ek[i] - d.mu_c) / d.W;
        f[3] = (ek[j] - d.mu_c) / d.W;
        f[4] = wn / wc;
        f[5] = n >= Nw_c ? 1.0 : 0.0;
        f[6] = i == j ? 1.0 : 0.0;
        f[7] = d.U / d.W;
        f[8] = d.J / d.W;
        f[9] = 100.0 * d.T / d.W;
        f[10] = d.fill / d.Norb;
        f[11] = d.stoner;
        f[12] = d.W / (d.W + wn);
        f[13] = s0.x / d.s_scale;
        f[14] = s0.y / d.s_scale;
        f[15] = 0.0;
        const long long r = (p * No + i) * No + j;
        __nv_bfloat16* xr = X + r * kLwsNF;
#pragma unroll
        for (int q = 0; q < kLwsNF; ++q) xr[q] = __float2bfloat16_rn((float)f[q]);
        if (T) {
          T[2 * r] = (float)(sd.x / d.s_scale);
          T[2 * r + 1] = (float)(sd.y / d.s_scale);
        }
      }
    }
  }
}

__global__ void k_lws_to_bf16(__nv_bfloat16* __restrict__ out, const float* __restrict__ in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}

__global__ void k_lws_to_float(float* __restrict__ out, const __nv_bfloat16* __restrict__ in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = __bfloat162float(in[i]);
}

// -------------------------------------------------------------- network --
// One thread per row, parameters in shared memory (every lane reads the same
// weight at the same time: a broadcast).  Layer 1 is produced one unit at a
// time and added into the 64 layer-2 sums at once, so that only those sums
// live in registers; each sum still runs over the units in order.  H1/H2
// (the stored activations) are written when non-null.
__global__ void __launch_bounds__(kThr) k_lws_forward(const __nv_bfloat16* __restrict__ X,
                                                      const float* __restrict__ theta, float* __restrict__ Y,
                                                      __nv_bfloat16* __restrict__ H1, __nv_bfloat16* __restrict__ H2,
                                                      long long M) {
  __shared__ float sp[kLwsNParam];
  for (int i = threadIdx.x; i < kLwsNParam; i += blockDim.x) sp[i] = theta[i];
  __syncthreads();
  const float* W1 = sp;
  const float* b1 = sp + kLwsOffB1;
  const float* W2 = sp + kLwsOffW2;
  const float* b2 = sp + kLwsOffB2;
  const float* W3 = sp + kLwsOffW3;
  const float* b3 = sp + kLwsOffB3;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x) {
    float x[kLwsNF];
#pragma unroll
    for (int q = 0; q < kLwsNF; ++q) x[q] = __bfloat162float(X[r * kLwsNF + q]);
    float z2[kLwsNH];
#pragma unroll
    for (int o = 0; o < kLwsNH; ++o) z2[o] = b2[o];
#pragma unroll 1
    for (int q = 0; q < kLwsNH; ++q) {
      float z = b1[q];
#pragma unroll
      for (int i = 0; i < kLwsNF; ++i) z = fmaf(W1[q * kLwsNF + i], x[i], z);
      const float h = bf16_round(tanhf(z));
      if (H1) H1[r * kLwsNH + q] = __float2bfloat16_rn(h);
#pragma unroll
      for (int o = 0; o < kLwsNH; ++o) z2[o] = fmaf(W2[o * kLwsNH + q], h, z2[o]);
    }
    float y0 = b3[0], y1 = b3[1];
#pragma unroll
    for (int o = 0; o < kLwsNH; ++o) {
      const float h = bf16_round(tanhf(z2[o]));
      if (H2) H2[r * kLwsNH + o] = __float2bfloat16_rn(h);
      y0 = fmaf(W3[o], h, y0);
      y1 = fmaf(W3[kLwsNH + o], h, y1);
    }
    Y[2 * r] = y0;
    Y[2 * r + 1] = y1;
  }
}

// Per row: dY = scale (y - t), dZ2 = (dY W3) (1 - h2^2), dZ1 = (dZ2 W2)
// (1 - h1^2); the block's sum of (y - t)^2 into lossp[blockIdx.x].  dZ2 is
// produced one unit at a time and added into the 64 sums of dZ2 W2.
__global__ void __launch_bounds__(kThr) k_lws_backward_rows(const float* __restrict__ Y, const float* __restrict__ T,
                                                            const __nv_bfloat16* __restrict__ H1,
                                                            const __nv_bfloat16* __restrict__ H2,
                                                            const float* __restrict__ theta, float* __restrict__ DY,
                                                            float* __restrict__ DZ2, float* __restrict__ DZ1,
                                                            double* __restrict__ lossp, long long M, float scale) {
  __shared__ float W2s[kLwsNH * kLwsNH];
  __shared__ float W3s[kLwsNO * kLwsNH];
  __shared__ double red[kThr];
  for (int i = threadIdx.x; i < kLwsNH * kLwsNH; i += blockDim.x) W2s[i] = theta[kLwsOffW2 + i];
  for (int i = threadIdx.x; i < kLwsNO * kLwsNH; i += blockDim.x) W3s[i] = theta[kLwsOffW3 + i];
  __syncthreads();
  double loss = 0.0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < M; r += (long long)gridDim.x * blockDim.x) {
    const float d0 = Y[2 * r] - T[2 * r], d1 = Y[2 * r + 1] - T[2 * r + 1];
    loss += (double)d0 * d0 + (double)d1 * d1;
    const float dy0 = scale * d0, dy1 = scale * d1;
    DY[2 * r] = dy0;
    DY[2 * r + 1] = dy1;
    float dh[kLwsNH];
#pragma unroll
    for (int i = 0; i < kLwsNH; ++i) dh[i] = 0.f;
#pragma unroll 1
    for (int o = 0; o < kLwsNH; ++o) {
      const float h = __bfloat162float(H2[r * kLwsNH + o]);
      const float dz2 = (W3s[o] * dy0 + W3s[kLwsNH + o] * dy1) * (1.f - h * h);
      DZ2[r * kLwsNH + o] = dz2;
#pragma unroll
      for (int i = 0; i < kLwsNH; ++i) dh[i] = fmaf(W2s[o * kLwsNH + i], dz2, dh[i]);
    }
#pragma unroll
    for (int i = 0; i < kLwsNH; ++i) {
      const float h = __bfloat162float(H1[r * kLwsNH + i]);
      DZ1[r * kLwsNH + i] = dh[i] * (1.f - h * h);
    }
  }
  red[threadIdx.x] = loss;
  __syncthreads();
  for (int s = kThr / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) lossp[blockIdx.x] = red[0];
}

// Weight and bias gradients of one layer as partial sums over row chunks:
// part[c][i * NB + j] = sum over the chunk's rows of A[r][i] B[r][j] and
// part[c][NA * NB + i] = sum of A[r][i].  The layout [W (NA x NB), b (NA)]
// is the layer's own segment of the flat parameter vector.
template <int NA, int NB>
__global__ void __launch_bounds__(kThr) k_lws_outer(float* __restrict__ part, const float* __restrict__ A,
                                                    const __nv_bfloat16* __restrict__ B, long long M, long long rpc) {
  constexpr int NOUT = NA * NB + NA;
  constexpr int PER = (NOUT + kThr - 1) / kThr;
  constexpr int TR = 32;
  __shared__ float As[TR][NA];
  __shared__ float Bs[TR][NB];
  float acc[PER];
#pragma unroll
  for (int s = 0; s < PER; ++s) acc[s] = 0.f;
  const long long r0 = (long long)blockIdx.x * rpc;
  const long long r1 = r0 + rpc < M ? r0 + rpc : M;
  for (long long base = r0; base < r1; base += TR) {
    const int nt = (int)((r1 - base) < TR ? (r1 - base) : TR);
    for (int q = threadIdx.x; q < TR * NA; q += blockDim.x) {
      const int t = q / NA, i = q % NA;
      As[t][i] = t < nt ? A[(base + t) * NA + i] : 0.f;
    }
    for (int q = threadIdx.x; q < TR * NB; q += blockDim.x) {
      const int t = q / NB, j = q % NB;
      Bs[t][j] = t < nt ? __bfloat162float(B[(base + t) * NB + j]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < PER; ++s) {
      const int o = threadIdx.x + kThr * s;
      if (o < NA * NB) {
        const int i = o / NB, j = o % NB;
        float a = acc[s];
        for (int t = 0; t < TR; ++t) a = fmaf(As[t][i], Bs[t][j], a);
        acc[s] = a;
      } else if (o < NOUT) {
        const int i = o - NA * NB;
        float a = acc[s];
        for (int t = 0; t < TR; ++t) a += As[t][i];
        acc[s] = a;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < PER; ++s) {
    const int o = threadIdx.x + kThr * s;
    if (o < NOUT) part[(long long)blockIdx.x * NOUT + o] = acc[s];
  }
}

// grad[o] (+)= sum over chunks in order: deterministic for a given chunking
__global__ void k_lws_reduce(float* __restrict__ grad, const float* __restrict__ part, int nout, int nchunks,
                             int accumulate) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < nout; o += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < nchunks; ++c) s += part[(long long)c * nout + o];
    grad[o] = accumulate ? grad[o] + s : s;
  }
}

// Adam (Kingma and Ba 2015) with bias correction, each operation rounded on
// its own (no contraction into fused multiply-adds).
__global__ void k_lws_adam(float* __restrict__ theta, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, int n, float lr, float b1, float omb1, float b2, float omb2,
                           float eps, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = __fadd_rn(__fmul_rn(b1, m[i]), __fmul_rn(omb1, gi));
    const float vi = __fadd_rn(__fmul_rn(b2, v[i]), __fmul_rn(__fmul_rn(omb2, gi), gi));
    const float mh = __fdiv_rn(mi, bc1), vh = __fdiv_rn(vi, bc2);
    theta[i] = __fsub_rn(theta[i], __fdiv_rn(__fmul_rn(lr, mh), __fadd_rn(__fsqrt_rn(vh), eps)));
    m[i] = mi;
    v[i] = vi;
  }
}

__global__ void k_lws_gather(__nv_bfloat16* __restrict__ Xb, float* __restrict__ Tb, const __nv_bfloat16* __restrict__ X,
                             const float* __restrict__ T, const long long* __restrict__ idx, long long B) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < B; r += (long long)gridDim.x * blockDim.x) {
    const long long s = idx[r];
#pragma unroll
    for (int q = 0; q < kLwsNF; ++q) Xb[r * kLwsNF + q] = X[s * kLwsNF + q];
    Tb[2 * r] = T[2 * s];
    Tb[2 * r + 1] = T[2 * s + 1];
  }
}

// Sigma(k, n) += U (s (y0 + i y1))_ij U^dagger for the pairs p0 .. p0+P-1
// (pair p = k + Nk n); Y holds the chunk's rows [P][No][No][2].
__global__ void k_lws_apply(double2* __restrict__ sig, const double2* __restrict__ U, const float* __restrict__ Y,
                            long long p0, long long P, int Nk, int Nw, int No, double s) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P;
       p += (long long)gridDim.x * blockDim.x) {
    const long long k = (p0 + p) % Nk, n = (p0 + p) / Nk;
    const double2* Uk = U + (long long)No * No * k;
    const float* y = Y + 2 * p * No * No;
    for (int b = 0; b < No; ++b) {
      double2 t[kMaxNo];
      for (int i = 0; i < No; ++i) {
        double2 acc = make_double2(0, 0);
        for (int j = 0; j < No; ++j) {
          const double2 dy = make_double2(s * (double)y[2 * (i * No + j)], s * (double)y[2 * (i * No + j) + 1]);
          acc = zadd(acc, zmulc(dy, Uk[b + No * j]));
        }
        t[i] = acc;
      }
      for (int a = 0; a < No; ++a) {
        double2 acc = make_double2(0, 0);
        for (int i = 0; i < No; ++i) acc = zadd(acc, zmul(Uk[a + No * i], t[i]));
        const long long e = sidx(k, n, a, b, Nk, Nw, No);
        sig[e] = zadd(sig[e], acc);
      }
    }
  }
}

// --------------------------------------------------------------- host ----
std::mutex g_lws_mu;
std::vector<std::unique_ptr<LwsNet>> g_lws;

void check_desc(const LwsDesc& d, int No) {
  PGB_CHECK(std::isfinite(d.W) && d.W > 0, "band width W must be positive");
  PGB_CHECK(std::isfinite(d.s_scale) && d.s_scale > 0, "s_scale = max |Sigma_seed| must be positive");
  PGB_CHECK(d.T > 0, "temperature must be positive");
  PGB_CHECK((int)std::lround(d.Norb) == No, "desc Norb differs from Norb");
}

void check_shape(int Nk, int Nw, int Nw_c, int No) {
  PGB_CHECK(No >= 1 && No <= kMaxNo, "the learned warm start takes 1 to 8 orbitals");
  PGB_CHECK(Nk >= 1 && Nw >= 1, "empty mesh");
  PGB_CHECK(Nw_c >= 1 && Nw_c <= Nw, "the coarse Matsubara count must be in [1, Nw]");
}

// Device copies of one solution's arrays and of its pair list.
struct SolutionDev {
  DBuf<double2> ss, sf, U;
  DBuf<double> eig;
  DBuf<long long> kn;
};

void upload_solution(SolutionDev& s, const double2* sig_seed, const double2* sig_fine, const double2* uni,
                     const double* eig, const int64_t* kn, long long P, int Nk, int Nw, int No) {
  const size_t ns = (size_t)Nk * Nw * No * No;
  s.ss.alloc(ns);
  s.ss.upload(sig_seed, ns);
  if (sig_fine) {
    s.sf.alloc(ns);
    s.sf.upload(sig_fine, ns);
  }
  s.U.alloc((size_t)No * No * Nk);
  s.U.upload(uni, (size_t)No * No * Nk);
  s.eig.alloc((size_t)No * Nk);
  s.eig.upload(eig, (size_t)No * Nk);
  if (kn) {
    for (long long p = 0; p < P; ++p)
      PGB_CHECK(kn[2 * p] >= 0 && kn[2 * p] < Nk && kn[2 * p + 1] >= 0 && kn[2 * p + 1] < Nw,
                "a (k, n) pair lies outside the mesh");
    s.kn.alloc((size_t)2 * P);
    s.kn.upload(kn, (size_t)2 * P);
  }
}

void launch_features(__nv_bfloat16* X, float* T, const SolutionDev& s, long long p0, long long P, int Nk, int Nw,
                     int Nw_c, int No, const LwsDesc& d) {
  k_lws_features<<<blocks_for(P, 128, 1 << 20), 128, 0, ctx().stream>>>(
      X, T, s.ss.p, s.sf.p, s.U.p, s.eig.p, s.kn.p, p0, P, Nk, Nw, Nw_c, No, d);
  launched("lws_features");
}

// Scratch of one pass over up to `rows` rows.
struct Work {
  DBuf<float> Y, DY, DZ1, DZ2, part, grad, Tb;
  DBuf<__nv_bfloat16> H1, H2, Xb;
  DBuf<double> lossp;
  DBuf<long long> idx;
  int nblk = 0, nchunk = 0;
  explicit Work(long long rows, bool gather) {
    Y.alloc(2 * rows);
    DY.alloc(2 * rows);
    DZ1.alloc(kLwsNH * rows);
    DZ2.alloc(kLwsNH * rows);
    H1.alloc(kLwsNH * rows);
    H2.alloc(kLwsNH * rows);
    nblk = (int)std::min<long long>(blocks_for(rows, kThr, 1LL << 30), 4LL * std::max(1, ctx().num_sms));
    nchunk = (int)std::min<long long>((rows + 63) / 64, 2LL * std::max(1, ctx().num_sms));
    if (nchunk < 1) nchunk = 1;
    lossp.alloc(nblk);
    part.alloc((size_t)nchunk * (kLwsNH * kLwsNH + kLwsNH));
    grad.alloc(kLwsNParam);
    if (gather) {
      Xb.alloc(kLwsNF * rows);
      Tb.alloc(2 * rows);
      idx.alloc(rows);
    }
  }
};

template <int NA, int NB>
void layer_grad(Work& w, float* grad_seg, const float* A, const __nv_bfloat16* B, long long M, bool accumulate) {
  const long long rpc = (M + w.nchunk - 1) / w.nchunk;
  constexpr int nout = NA * NB + NA;
  k_lws_outer<NA, NB><<<w.nchunk, kThr, 0, ctx().stream>>>(w.part.p, A, B, M, rpc);
  launched("lws_outer");
  k_lws_reduce<<<blocks_for(nout, kThr, 64), kThr, 0, ctx().stream>>>(grad_seg, w.part.p, nout, w.nchunk,
                                                                        accumulate ? 1 : 0);
  launched("lws_reduce");
}

// forward + backward of M rows into w.grad (added when accumulate); returns
// the sum of squared errors
double pass(LwsNet& net, Work& w, const __nv_bfloat16* X, const float* T, long long M, float scale, bool accumulate) {
  cudaStream_t st = ctx().stream;
  const unsigned nb = (unsigned)std::min<long long>(blocks_for(M, kThr, 1LL << 30), w.nblk);
  k_lws_forward<<<nb, kThr, 0, st>>>(X, net.theta.p, w.Y.p, w.H1.p, w.H2.p, M);
  launched("lws_forward");
  w.lossp.zero();
  k_lws_backward_rows<<<nb, kThr, 0, st>>>(w.Y.p, T, w.H1.p, w.H2.p, net.theta.p, w.DY.p, w.DZ2.p, w.DZ1.p,
                                           w.lossp.p, M, scale);
  launched("lws_backward_rows");
  layer_grad<kLwsNH, kLwsNF>(w, w.grad.p, w.DZ1.p, X, M, accumulate);
  layer_grad<kLwsNH, kLwsNH>(w, w.grad.p + kLwsOffW2, w.DZ2.p, w.H1.p, M, accumulate);
  layer_grad<kLwsNO, kLwsNH>(w, w.grad.p + kLwsOffW3, w.DY.p, w.H2.p, M, accumulate);
  std::vector<double> lp(nb);
  w.lossp.download(lp.data(), nb);
  sync();
  double s = 0;
  for (double v : lp) s += v;
  return s;
}

void adam(LwsNet& net, const float* grad, double lr, double beta1, double beta2, double eps) {
  net.step += 1;
  const double t = (double)net.step;
  k_lws_adam<<<blocks_for(kLwsNParam, kThr, 64), kThr, 0, ctx().stream>>>(
      net.theta.p, net.m.p, net.v.p, grad, kLwsNParam, (float)lr, (float)beta1, (float)(1.0 - beta1), (float)beta2,
      (float)(1.0 - beta2), (float)eps, (float)(1.0 - std::pow(beta1, t)), (float)(1.0 - std::pow(beta2, t)));
  launched("lws_adam");
}

}  // namespace

int64_t lws_create() {
  ensure_context();
  auto net = std::make_unique<LwsNet>();
  net->theta.alloc(kLwsNParam);
  net->m.alloc(kLwsNParam);
  net->v.alloc(kLwsNParam);
  net->theta.zero();
  net->m.zero();
  net->v.zero();
  sync();
  std::lock_guard<std::mutex> lk(g_lws_mu);
  g_lws.push_back(std::move(net));
  return (int64_t)g_lws.size();
}

void lws_destroy(int64_t h) {
  std::lock_guard<std::mutex> lk(g_lws_mu);
  if (h >= 1 && h <= (int64_t)g_lws.size()) g_lws[h - 1].reset();
}

LwsNet& lws_get(int64_t h) {
  std::lock_guard<std::mutex> lk(g_lws_mu);
  PGB_CHECK(h >= 1 && h <= (int64_t)g_lws.size() && g_lws[h - 1], "unknown learned-warm-start handle");
  return *g_lws[h - 1];
}

void lws_set_params(LwsNet& net, const float* host, long long n) {
  PGB_CHECK(n == kLwsNParam, "the network has 5378 parameters");
  net.theta.upload(host, n);
  net.m.zero();
  net.v.zero();
  net.step = 0;
  sync();
}

void lws_get_params(LwsNet& net, float* host, long long n) {
  PGB_CHECK(n == kLwsNParam, "the network has 5378 parameters");
  net.theta.download(host, n);
  sync();
}

void lws_add_samples(LwsNet& net, const double2* sig_seed, const double2* sig_fine, const double2* uni,
                     const double* eig, const int64_t* kn, long long P, int Nk, int Nw, int Nw_c, int No,
                     const LwsDesc& d) {
  check_shape(Nk, Nw, Nw_c, No);
  check_desc(d, No);
  PGB_CHECK(sig_fine != nullptr, "training samples need the fine Sigma");
  PGB_CHECK(P >= 1, "no (k, n) pairs given");
  SolutionDev s;
  upload_solution(s, sig_seed, sig_fine, uni, eig, kn, P, Nk, Nw, No);
  const long long R = P * No * No;
  if (net.M + R > net.cap) {
    const long long cap = std::max(net.M + R, 2 * net.cap);
    DBuf<__nv_bfloat16> X(kLwsNF * cap);
    DBuf<float> T(2 * cap);
    if (net.M) {
      PGB_CUDA(cudaMemcpyAsync(X.p, net.X.p, sizeof(__nv_bfloat16) * kLwsNF * net.M, cudaMemcpyDeviceToDevice,
                               ctx().stream));
      PGB_CUDA(cudaMemcpyAsync(T.p, net.T.p, sizeof(float) * 2 * net.M, cudaMemcpyDeviceToDevice, ctx().stream));
    }
    net.X = std::move(X);
    net.T = std::move(T);
    net.cap = cap;
  }
  launch_features(net.X.p + kLwsNF * net.M, net.T.p + 2 * net.M, s, 0, P, Nk, Nw, Nw_c, No, d);
  net.M += R;
  sync();
}

void lws_clear_samples(LwsNet& net) {
  net.X.release();
  net.T.release();
  net.M = net.cap = 0;
  sync();
}

void lws_features_host(float* x, float* t, const double2* sig_seed, const double2* sig_fine, const double2* uni,
                       const double* eig, const int64_t* kn, long long P, int Nk, int Nw, int Nw_c, int No,
                       const LwsDesc& d) {
  ensure_context();
  check_shape(Nk, Nw, Nw_c, No);
  check_desc(d, No);
  PGB_CHECK(P >= 1, "no (k, n) pairs given");
  SolutionDev s;
  upload_solution(s, sig_seed, sig_fine, uni, eig, kn, P, Nk, Nw, No);
  const long long R = P * No * No;
  DBuf<__nv_bfloat16> X(kLwsNF * R);
  DBuf<float> T(sig_fine ? 2 * R : 0), Xf(kLwsNF * R);
  launch_features(X.p, sig_fine ? T.p : nullptr, s, 0, P, Nk, Nw, Nw_c, No, d);
  k_lws_to_float<<<blocks_for(kLwsNF * R, kThr, 1 << 16), kThr, 0, ctx().stream>>>(Xf.p, X.p, kLwsNF * R);
  launched("lws_to_float");
  Xf.download(x, kLwsNF * R);
  if (sig_fine && t) T.download(t, 2 * R);
  sync();
}

void lws_forward_host(LwsNet& net, const float* x, long long M, float* y) {
  PGB_CHECK(M >= 1, "no rows given");
  DBuf<float> xf(kLwsNF * M), Y(2 * M);
  DBuf<__nv_bfloat16> X(kLwsNF * M);
  xf.upload(x, kLwsNF * M);
  k_lws_to_bf16<<<blocks_for(kLwsNF * M, kThr, 1 << 16), kThr, 0, ctx().stream>>>(X.p, xf.p, kLwsNF * M);
  launched("lws_to_bf16");
  k_lws_forward<<<blocks_for(M, kThr, 1LL << 20), kThr, 0, ctx().stream>>>(X.p, net.theta.p, Y.p, nullptr, nullptr,
                                                                            M);
  launched("lws_forward");
  Y.download(y, 2 * M);
  sync();
}

double lws_loss_grad(LwsNet& net, float* grad) {
  PGB_CHECK(net.M >= 1, "the training set is empty");
  const long long B = std::min(net.M, kBatchRows);
  Work w(B, false);
  const float scale = (float)(2.0 / (double)net.M);
  double sse = 0;
  for (long long r0 = 0; r0 < net.M; r0 += B) {
    const long long n = std::min(B, net.M - r0);
    sse += pass(net, w, net.X.p + kLwsNF * r0, net.T.p + 2 * r0, n, scale, r0 > 0);
  }
  if (grad) {
    w.grad.download(grad, kLwsNParam);
    sync();
  }
  return sse / (double)net.M;
}

void lws_step_full(LwsNet& net, double lr, double beta1, double beta2, double eps, double* loss) {
  PGB_CHECK(net.M >= 1, "the training set is empty");
  const long long B = std::min(net.M, kBatchRows);
  Work w(B, false);
  const float scale = (float)(2.0 / (double)net.M);
  double sse = 0;
  for (long long r0 = 0; r0 < net.M; r0 += B) {
    const long long n = std::min(B, net.M - r0);
    sse += pass(net, w, net.X.p + kLwsNF * r0, net.T.p + 2 * r0, n, scale, r0 > 0);
  }
  adam(net, w.grad.p, lr, beta1, beta2, eps);
  sync();
  if (loss) *loss = sse / (double)net.M;
}

void lws_train(LwsNet& net, long long steps, long long batch, double lr, double beta1, double beta2, double eps,
               uint64_t seed, double* loss_out) {
  PGB_CHECK(net.M >= 1, "the training set is empty");
  PGB_CHECK(batch >= 1 && steps >= 0, "batch must be positive");
  Work w(batch, true);
  std::mt19937_64 rng(seed);
  std::uniform_int_distribution<long long> pick(0, net.M - 1);
  std::vector<long long> idx(batch);
  const float scale = (float)(2.0 / (double)batch);
  for (long long s = 0; s < steps; ++s) {
    for (auto& i : idx) i = pick(rng);
    w.idx.upload(idx.data(), batch);
    k_lws_gather<<<blocks_for(batch, kThr, 1 << 16), kThr, 0, ctx().stream>>>(w.Xb.p, w.Tb.p, net.X.p, net.T.p,
                                                                               w.idx.p, batch);
    launched("lws_gather");
    const double sse = pass(net, w, w.Xb.p, w.Tb.p, batch, scale, false);
    adam(net, w.grad.p, lr, beta1, beta2, eps);
    if (loss_out) loss_out[s] = sse / (double)batch;
  }
  sync();
}

void lws_apply(LwsNet& net, double2* sigma, const double2* uni, const double* eig, int Nk, int Nw, int Nw_c, int No,
               const LwsDesc& d) {
  check_shape(Nk, Nw, Nw_c, No);
  check_desc(d, No);
  SolutionDev s;
  upload_solution(s, sigma, nullptr, uni, eig, nullptr, 0, Nk, Nw, No);
  const long long P = (long long)Nk * Nw;
  const long long Pc = std::max<long long>(1, std::min<long long>(P, (32LL << 20) / ((long long)No * No)));
  DBuf<__nv_bfloat16> X(kLwsNF * Pc * No * No);
  DBuf<float> Y(2 * Pc * No * No);
  // the correction is added to a copy, so that every chunk reads the seed
  DBuf<double2> out((size_t)Nk * Nw * No * No);
  PGB_CUDA(cudaMemcpyAsync(out.p, s.ss.p, sizeof(double2) * Nk * Nw * No * No, cudaMemcpyDeviceToDevice,
                           ctx().stream));
  for (long long p0 = 0; p0 < P; p0 += Pc) {
    const long long n = std::min(Pc, P - p0), R = n * No * No;
    launch_features(X.p, nullptr, s, p0, n, Nk, Nw, Nw_c, No, d);
    k_lws_forward<<<blocks_for(R, kThr, 1LL << 20), kThr, 0, ctx().stream>>>(X.p, net.theta.p, Y.p, nullptr,
                                                                              nullptr, R);
    launched("lws_forward");
    k_lws_apply<<<blocks_for(n, 128, 1 << 20), 128, 0, ctx().stream>>>(out.p, s.U.p, Y.p, p0, n, Nk, Nw, No,
                                                                       d.s_scale);
    launched("lws_apply");
  }
  out.download(sigma, (size_t)Nk * Nw * No * No);
  sync();
}

}  // namespace pgb
