// Common device/host helpers of the GB300 FLEX engine: complex arithmetic on
// float2/double2, error reporting, the per-process CUDA context.
#pragma once

#include <atomic>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace pgb {

// ---------------------------------------------------------------- complex --
template <typename R> struct cvec;
template <> struct cvec<float> { using type = float2; };
template <> struct cvec<double> { using type = double2; };
template <typename R> using cx = typename cvec<R>::type;

__host__ __device__ __forceinline__ float2 mkc(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mkc(double a, double b) { return make_double2(a, b); }
template <typename R> __host__ __device__ __forceinline__ cx<R> cmk(R a, R b) { return mkc(a, b); }

__host__ __device__ __forceinline__ float2 operator+(float2 a, float2 b) { return mkc(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 operator+(double2 a, double2 b) { return mkc(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a, float2 b) { return mkc(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 operator-(double2 a, double2 b) { return mkc(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a) { return mkc(-a.x, -a.y); }
__host__ __device__ __forceinline__ double2 operator-(double2 a) { return mkc(-a.x, -a.y); }
__host__ __device__ __forceinline__ float2 operator*(float2 a, float2 b) {
  return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 operator*(double2 a, double2 b) {
  return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 operator*(float a, float2 b) { return mkc(a * b.x, a * b.y); }
__host__ __device__ __forceinline__ double2 operator*(double a, double2 b) { return mkc(a * b.x, a * b.y); }
__host__ __device__ __forceinline__ float2 operator*(float2 b, float a) { return mkc(a * b.x, a * b.y); }
__host__ __device__ __forceinline__ double2 operator*(double2 b, double a) { return mkc(a * b.x, a * b.y); }
__host__ __device__ __forceinline__ float2& operator+=(float2& a, float2 b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ double2& operator+=(double2& a, double2 b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ float2& operator-=(float2& a, float2 b) { a.x -= b.x; a.y -= b.y; return a; }
__host__ __device__ __forceinline__ double2& operator-=(double2& a, double2 b) { a.x -= b.x; a.y -= b.y; return a; }

__host__ __device__ __forceinline__ float2 conj(float2 a) { return mkc(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 conj(double2 a) { return mkc(a.x, -a.y); }
__host__ __device__ __forceinline__ float abs2(float2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }
// a * (s i), s = +-1
__host__ __device__ __forceinline__ float2 muli(float2 a, float s) { return mkc(-s * a.y, s * a.x); }
__host__ __device__ __forceinline__ double2 muli(double2 a, double s) { return mkc(-s * a.y, s * a.x); }
// complex division a / b (scaled to avoid overflow for large |b|)
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  double s = fabs(b.x) + fabs(b.y);
  double bx = b.x / s, by = b.y / s;
  double d = bx * bx + by * by;
  double ax = a.x / s, ay = a.y / s;
  return mkc((ax * bx + ay * by) / d, (ay * bx - ax * by) / d);
}
__host__ __device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
  float s = fabsf(b.x) + fabsf(b.y);
  float bx = b.x / s, by = b.y / s;
  float d = bx * bx + by * by;
  float ax = a.x / s, ay = a.y / s;
  return mkc((ax * bx + ay * by) / d, (ay * bx - ax * by) / d);
}
__host__ __device__ __forceinline__ double cabs_(double2 a) { return hypot(a.x, a.y); }
__host__ __device__ __forceinline__ float cabs_(float2 a) { return hypotf(a.x, a.y); }

template <typename D, typename S> __host__ __device__ __forceinline__ cx<D> ccast(S a) {
  return cmk<D>((D)a.x, (D)a.y);
}

// ------------------------------------------------------------ double-float --
// A real carried as the unevaluated sum hi + lo of two floats (|lo| at most
// half an ulp of hi): about 48 significant bits, with all arithmetic on the
// FP32 pipe, which on GB300 has 64 times the FP64 rate.  The add and multiply
// are the double-word algorithms built from Knuth's two-sum and the FMA
// two-product (Dekker 1971; Hida, Li and Bailey, "Algorithms for quad-double
// precision floating point arithmetic", ARITH 2001).  The FFT convolutions of the FLEX
// loop use it where FP32 rounding would set the residual's floor.
struct dfl {
  float hi, lo;
  __host__ __device__ constexpr dfl() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dfl(float f) : hi(f), lo(0.f) {}
  __host__ __device__ constexpr dfl(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr dfl(int i) : dfl((double)i) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
struct __align__(16) cdf {
  dfl x, y;
};
template <> struct cvec<dfl> { using type = cdf; };

__host__ __device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfl(s, (a - (s - bb)) + (b - bb));
}
__host__ __device__ __forceinline__ dfl fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return dfl(s, b - (s - a));
}
// Dekker's add2: the error is bounded by a few 2^-48 (|a| + |b|) rather than
// by |a + b|, which is the normwise bound an FFT or a contraction needs
// (measured 8e-15 against 7e-15 for the 20-flop accurate add); 11 flops.
__host__ __device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__host__ __device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { a = a + b; return a; }
__host__ __device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { a = a - b; return a; }
__host__ __device__ __forceinline__ dfl dabs(dfl a) { return a.hi < 0.f ? -a : a; }
__host__ __device__ __forceinline__ bool operator<(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
// |x| < t for each bulk type (the reference's small-part zeroing)
__host__ __device__ __forceinline__ bool abs_below(float x, double t) { return fabsf(x) < (float)t; }
__host__ __device__ __forceinline__ bool abs_below(double x, double t) { return fabs(x) < t; }
__host__ __device__ __forceinline__ bool abs_below(dfl x, double t) { return dabs(x) < dfl(t); }

__host__ __device__ __forceinline__ cdf mkc(dfl a, dfl b) {
  cdf r;
  r.x = a;
  r.y = b;
  return r;
}
__host__ __device__ __forceinline__ cdf operator+(cdf a, cdf b) { return mkc(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cdf operator-(cdf a, cdf b) { return mkc(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cdf operator-(cdf a) { return mkc(-a.x, -a.y); }
// a*b + c*d as one double-word sum of the two double-word products, with one
// renormalization (19 flops against 25 for two renormalized products and
// Dekker's sum); the complex product's two components
__host__ __device__ __forceinline__ dfl dot2(dfl a, dfl b, dfl c, dfl d) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float q = c.hi * d.hi;
  float f = fmaf(c.hi, d.hi, -q);
  f = fmaf(c.hi, d.lo, fmaf(c.lo, d.hi, f));
  const dfl s = two_sum(p, q);
  return fast_two_sum(s.hi, s.lo + (e + f));
}
__host__ __device__ __forceinline__ cdf operator*(cdf a, cdf b) {
  return mkc(dot2(a.x, b.x, -a.y, b.y), dot2(a.x, b.y, a.y, b.x));
}
__host__ __device__ __forceinline__ cdf operator*(dfl s, cdf b) { return mkc(s * b.x, s * b.y); }
__host__ __device__ __forceinline__ cdf operator*(cdf b, dfl s) { return mkc(s * b.x, s * b.y); }
__host__ __device__ __forceinline__ cdf& operator+=(cdf& a, cdf b) { a = a + b; return a; }
__host__ __device__ __forceinline__ cdf& operator-=(cdf& a, cdf b) { a = a - b; return a; }
__host__ __device__ __forceinline__ cdf conj(cdf a) { return mkc(a.x, -a.y); }
// a * (s i), s = +-1 (a sign change, no rounding)
__host__ __device__ __forceinline__ cdf muli(cdf a, dfl s) { return s.hi > 0.f ? mkc(-a.y, a.x) : mkc(a.y, -a.x); }

// Comparisons, division and the helpers the warp Gauss-Jordan elimination
// uses for every bulk type (mad = multiply-add: one rounding in float and
// double, the double-float product and sum otherwise).
__host__ __device__ __forceinline__ bool operator>(dfl a, dfl b) { return b < a; }
__host__ __device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
// Dekker's division: a float quotient, the double-float remainder a - b q1,
// one float correction
__host__ __device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = a.hi / b.hi;
  const dfl r = a - b * dfl(q1);
  const float q2 = r.hi / b.hi;
  return fast_two_sum(q1, q2);
}
__host__ __device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
__host__ __device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
// a*b + c with one renormalization: the double-word product's high word and
// error term go straight into Dekker's sum with c (15 flops against 18 for
// the renormalized product plus the sum; same error bound, a few 2^-47)
__host__ __device__ __forceinline__ dfl mad(dfl a, dfl b, dfl c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const dfl s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, s.lo + (e + c.lo));
}
__host__ __device__ __forceinline__ dfl cabs1(cdf a) { return dabs(a.x) + dabs(a.y); }
__host__ __device__ __forceinline__ cdf cdiv(cdf a, cdf b) {  // same scaling as the double version
  const dfl s = dabs(b.x) + dabs(b.y);
  const dfl bx = b.x / s, by = b.y / s;
  const dfl d = bx * bx + by * by;
  const dfl ax = a.x / s, ay = a.y / s;
  return mkc((ax * bx + ay * by) / d, (ay * bx - ax * by) / d);
}
// 1 / b as conj(b) / |b|^2: one real division instead of cdiv's six, for
// |b|^2 well inside the type's range (else cdiv's scaled form)
__host__ __device__ __forceinline__ float2 crecip(float2 b) {
  const float d = fmaf(b.x, b.x, b.y * b.y);
  if (!(d > 1e-30f && d < 1e30f)) return cdiv(mkc(1.f, 0.f), b);
  const float r = 1.0f / d;
  return mkc(b.x * r, -b.y * r);
}
__host__ __device__ __forceinline__ double2 crecip(double2 b) {
  const double d = fma(b.x, b.x, b.y * b.y);
  if (!(d > 1e-280 && d < 1e280)) return cdiv(mkc(1.0, 0.0), b);
  const double r = 1.0 / d;
  return mkc(b.x * r, -b.y * r);
}
__host__ __device__ __forceinline__ cdf crecip(cdf b) {
  const dfl d = b.x * b.x + b.y * b.y;
  if (!(d.hi > 1e-30f && d.hi < 1e30f)) return cdiv(mkc(dfl(1.f), dfl(0.f)), b);
  const dfl r = dfl(1.f) / d;
  return mkc(b.x * r, -(b.y * r));
}
#ifdef __CUDACC__
__device__ __forceinline__ float shfl_idx(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double shfl_idx(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ dfl shfl_idx(dfl v, int src) {
  return dfl(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ dfl shfl_xor(dfl v, int m) {
  return dfl(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}
#endif

// ---------------------------------------------------------------- errors --
struct Error : std::runtime_error {
  explicit Error(const std::string& s) : std::runtime_error(s) {}
};
// an argument or input file the caller has to fix (error code 2 at the ABI,
// ValueError in the Python wrappers); every other failure is code 1
struct BadInput : Error {
  explicit BadInput(const std::string& s) : Error(s) {}
};

#define PGB_CUDA(call)                                                               \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      throw ::pgb::Error(std::string(#call) + ": " + cudaGetErrorString(e_));        \
  } while (0)

// Raises a kernel's dynamic shared memory limit once per process (a
// function-local static, so the first call is thread-safe).  KERNEL goes in
// parentheses when it has template arguments.
#define PGB_SMEM_LIMIT_ONCE(KERNEL, BYTES)                                                               \
  do {                                                                                                   \
    static const bool pgb_smem_set_ = [&] {                                                              \
      PGB_CUDA(cudaFuncSetAttribute(KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(BYTES))); \
      return true;                                                                                       \
    }();                                                                                                 \
    (void)pgb_smem_set_;                                                                                 \
  } while (0)

#define PGB_CHECK(cond, msg)                     \
  do {                                           \
    if (!(cond)) throw ::pgb::Error(msg);        \
  } while (0)

// Device bytes this process can still allocate: what the driver reports free
// plus what the default memory pool holds but no longer uses (blocks freed with
// cudaFreeAsync stay in the pool, whose release threshold is kept at maximum).
inline size_t device_bytes_available() {
  size_t freeb = 0, totb = 0;
  if (cudaMemGetInfo(&freeb, &totb) != cudaSuccess) return 0;
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      freeb += (size_t)(reserved - used);
  }
  return freeb;
}

inline void launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(std::string("launch ") + what + ": " + cudaGetErrorString(e));
}

inline unsigned nblocks(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// -------------------------------------------------------------- context --
// One CUDA stream per context; every entry point of the library runs on its
// caller's context and synchronizes that stream before returning (the C ABI
// is synchronous like the reference's Fortran subroutines).  The process has
// one context; a host thread that calls pyrpa_gb_set_thread_stream(1) gets a
// context of its own (own stream, device error flags, launch counter and
// settings copied from the process context), so that several threads can
// solve independent problems at once and their kernels overlap on the GPU.
struct Context {
  cudaStream_t stream = nullptr;
  int device = 0;
  int num_sms = 0;
  bool ready = false;
  int precision = 64;          // 64: FP64 bulk; 32: complex FP32 bulk with FP64 steps; 3264: mixed FLEX schedule
  int verbose = 1;             // progress prints like the reference's stdout
  // 0: the reference's fixed Krylov size in lin_eliash; > 0: each Arnoldi pass
  // restarts from its Ritz vector until |h_{m+1,m} y_m| / |lambda| < tol
  double arnoldi_tol = 0.0;
  // bumped by the entry points, some of which run on callers' own threads
  std::atomic<long long> kernel_launches{0};
  // this context's slot of the device error flags that kernels raise
  // (singular matrices, unconverged eigenvalue iterations)
  int* err = nullptr;
  // this context's timeout flag of the TMA passes, in mapped pinned host
  // memory (made on first use)
  volatile int* tma_flag_h = nullptr;
  int* tma_flag_d = nullptr;
};
Context& ctx();
void ensure_context();
// device error flag slots: slot 0 is the process context's, the others go
// to thread contexts
constexpr int kErrSlots = 64;
int* err_slot_address(int slot);

// Device allocation through the stream-ordered pool (memory stays cached in
// the pool between calls, so repeated calls of one shape do not re-map HBM).
template <typename T> struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) PGB_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), ctx().stream));
  }
  void release() {
    if (p) cudaFreeAsync(p, ctx().stream);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
  size_t bytes() const { return n * sizeof(T); }
  void zero() {
    if (n) PGB_CUDA(cudaMemsetAsync(p, 0, bytes(), ctx().stream));
  }
  void upload(const void* h, size_t count) {
    PGB_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, ctx().stream));
  }
  void download(void* h, size_t count) const {
    PGB_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, ctx().stream));
  }
};

// throws if a TMA-staged FFT pass gave up a bounded wait since the last call
// (the flag is in mapped host memory: reading it costs no transfer)
void fft_raise_pending();
inline void sync() {
  PGB_CUDA(cudaStreamSynchronize(ctx().stream));
  fft_raise_pending();
}

void log(const char* fmt, ...);

}  // namespace pgb
