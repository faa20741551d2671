// Small dense complex linear algebra on the device, FP64 unless templated.
//
// Thread-level routines work on one row-major n x n matrix in local memory
// (n <= kMaxOrb): inverse by Gauss-Jordan with partial pivoting (the reference
// uses zgetrf+zgetri per (k,iw), fself.f90:138-157), eigenvalues of a general
// complex matrix by Householder Hessenberg reduction and single-shift QR with
// Wilkinson shifts (Golub & Van Loan, "Matrix Computations", 4th ed., 7.4-7.5;
// the reference calls zgeev, fself.f90:689-711 and fchi.f90:352-399), and
// eigen-decomposition of a Hermitian matrix by cyclic complex Jacobi
// rotations (the reference calls zheev, fmod.f90:209-248).
//
// Warp-level routines work on one n x n matrix (n <= 32) in shared memory with
// lane = row: products with a real matrix and an LU solve with partial
// pivoting for n right-hand sides (the reference calls zgemm/zgesv per (q,iv),
// fUJ.f90:253-365).  Pivots use |Re|+|Im| with the first maximum, as izamax.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int kMaxOrb = 8;
constexpr int kMaxChi = 32;

__host__ __device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
__host__ __device__ __forceinline__ float cabs1(float2 a) { return fabsf(a.x) + fabsf(a.y); }

// ---------------------------------------------------------------- thread --
// In-place inverse of row-major A (n x n).  Returns false if singular.
template <typename T>
__host__ __device__ bool inv_small(T* A, int n) {
  using Rt = decltype(cabs1(A[0]));
  int piv[kMaxOrb * 4];
  for (int k = 0; k < n; ++k) {
    int p = k;
    Rt best = cabs1(A[k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      Rt v = cabs1(A[i * n + k]);
      if (v > best) { best = v; p = i; }
    }
    piv[k] = p;
    if (best == 0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) { T t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
    T d = cdiv(cmk<Rt>(1, 0), A[k * n + k]);
    A[k * n + k] = cmk<Rt>(1, 0);
    for (int j = 0; j < n; ++j) A[k * n + j] = A[k * n + j] * d;
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      T f = A[i * n + k];
      A[i * n + k] = cmk<Rt>(0, 0);
      for (int j = 0; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
    }
  }
  // undo the row interchanges by column interchanges in reverse order
  for (int k = n - 1; k >= 0; --k) {
    const int p = piv[k];
    if (p != k)
      for (int i = 0; i < n; ++i) { T t = A[i * n + k]; A[i * n + k] = A[i * n + p]; A[i * n + p] = t; }
  }
  return true;
}

// complex sqrt (principal branch)
__host__ __device__ inline double2 csqrt_(double2 z) {
  double r = hypot(z.x, z.y);
  if (r == 0.0) return mkc(0.0, 0.0);
  double t = sqrt(0.5 * (r + fabs(z.x)));
  if (z.x >= 0) return mkc(t, z.y / (2 * t));
  return mkc(fabs(z.y) / (2 * t), z.y >= 0 ? t : -t);
}

// Eigenvalues of a general complex row-major matrix A (destroyed); w[n].
// Returns the number of QR sweeps, or -1 if the iteration did not converge.
__host__ __device__ inline int eigvals_general(double2* A, int n, double2* w) {
  // Householder reduction to upper Hessenberg form
  for (int k = 0; k + 2 < n; ++k) {
    double xn = 0;
    for (int i = k + 1; i < n; ++i) xn += abs2(A[i * n + k]);
    xn = sqrt(xn);
    if (xn == 0) continue;
    double2 x0 = A[(k + 1) * n + k];
    double a0 = hypot(x0.x, x0.y);
    double2 ph = a0 > 0 ? mkc(x0.x / a0, x0.y / a0) : mkc(1.0, 0.0);
    double2 alpha = mkc(-ph.x * xn, -ph.y * xn);
    // v = x - alpha e1 (stored in column k below the subdiagonal scratch)
    double2 v[64];
    for (int i = k + 1; i < n; ++i) v[i] = A[i * n + k];
    v[k + 1] = v[k + 1] - alpha;
    double vn = 0;
    for (int i = k + 1; i < n; ++i) vn += abs2(v[i]);
    if (vn == 0) continue;
    double sc = 2.0 / vn;
    // A = (I - sc v v^H) A  on rows k+1..n-1
    for (int j = k; j < n; ++j) {
      double2 s = mkc(0.0, 0.0);
      for (int i = k + 1; i < n; ++i) s += conj(v[i]) * A[i * n + j];
      s = sc * s;
      for (int i = k + 1; i < n; ++i) A[i * n + j] -= v[i] * s;
    }
    // A = A (I - sc v v^H) on columns k+1..n-1
    for (int i = 0; i < n; ++i) {
      double2 s = mkc(0.0, 0.0);
      for (int j = k + 1; j < n; ++j) s += A[i * n + j] * v[j];
      s = sc * s;
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= s * conj(v[j]);
    }
    for (int i = k + 2; i < n; ++i) A[i * n + k] = mkc(0.0, 0.0);
  }
  // shifted QR on the active block [lo, hi]
  int hi = n - 1, iter = 0, total = 0;
  const double eps = 2.220446049250313e-16;
  while (hi >= 0) {
    if (hi == 0) { w[0] = A[0]; break; }
    int l = hi;
    while (l > 0) {
      double s = cabs1(A[(l - 1) * n + l - 1]) + cabs1(A[l * n + l]);
      if (s == 0) s = 1.0;
      if (cabs1(A[l * n + l - 1]) <= eps * s) break;
      --l;
    }
    if (l == hi) {
      w[hi] = A[hi * n + hi];
      --hi;
      iter = 0;
      continue;
    }
    if (l > 0) A[l * n + l - 1] = mkc(0.0, 0.0);
    if (++iter > 60 || ++total > 60 * n) return -1;
    double2 mu;
    if (iter % 11 == 10) {
      // exceptional shift
      double e = cabs1(A[hi * n + hi - 1]) + (hi >= 2 ? cabs1(A[(hi - 1) * n + hi - 2]) : 0.0);
      mu = A[hi * n + hi] + mkc(0.75 * e, 0.0);
    } else {
      double2 a = A[(hi - 1) * n + hi - 1], b = A[(hi - 1) * n + hi];
      double2 c = A[hi * n + hi - 1], d = A[hi * n + hi];
      double2 hd = 0.5 * (a - d);
      double2 disc = csqrt_(hd * hd + b * c);
      double2 m1 = 0.5 * (a + d) + disc, m2 = 0.5 * (a + d) - disc;
      mu = (abs2(m1 - d) < abs2(m2 - d)) ? m1 : m2;
    }
    for (int i = l; i <= hi; ++i) A[i * n + i] -= mu;
    double cs[64];
    double2 sn[64];
    for (int k = l; k < hi; ++k) {
      double2 a = A[k * n + k], b = A[(k + 1) * n + k];
      double aa = hypot(a.x, a.y), bb = hypot(b.x, b.y);
      double r = hypot(aa, bb);
      double c;
      double2 s;
      if (r == 0) { c = 1.0; s = mkc(0.0, 0.0); }
      else if (aa == 0) { c = 0.0; s = conj(b) * (1.0 / bb); }
      else { c = aa / r; s = mkc(a.x / aa, a.y / aa) * conj(b) * (1.0 / r); }
      cs[k] = c;
      sn[k] = s;
      for (int j = k; j <= hi; ++j) {
        double2 x = A[k * n + j], y = A[(k + 1) * n + j];
        A[k * n + j] = c * x + s * y;
        A[(k + 1) * n + j] = c * y - conj(s) * x;
      }
    }
    for (int k = l; k < hi; ++k) {
      double c = cs[k];
      double2 s = sn[k];
      int imax = (k + 2 < hi) ? k + 2 : hi;
      for (int i = l; i <= imax; ++i) {
        double2 x = A[i * n + k], y = A[i * n + k + 1];
        A[i * n + k] = c * x + y * conj(s);
        A[i * n + k + 1] = c * y - x * s;
      }
    }
    for (int i = l; i <= hi; ++i) A[i * n + i] += mu;
  }
  return total;
}

// Hermitian eigen-decomposition by cyclic Jacobi: A row-major (destroyed),
// eigenvalues ascending in w, eigenvectors as columns of V (row-major).
__host__ __device__ inline void jacobi_herm(double2* A, int n, double* w, double2* V) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i * n + j] = mkc(i == j ? 1.0 : 0.0, 0.0);
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0, diag = 0;
    for (int i = 0; i < n; ++i) {
      diag += A[i * n + i].x * A[i * n + i].x;
      for (int j = i + 1; j < n; ++j) off += abs2(A[i * n + j]);
    }
    if (off <= 1e-32 * (diag + 1e-300)) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double2 b = A[p * n + q];
        double ab = hypot(b.x, b.y);
        if (ab < 1e-300) continue;
        double2 e = mkc(b.x / ab, b.y / ab);
        double theta = (A[q * n + q].x - A[p * n + p].x) / (2.0 * ab);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        // U = D J: U_pp = c, U_pq = s, U_qp = -s conj(e), U_qq = c conj(e)
        double2 upp = mkc(c, 0.0), upq = mkc(s, 0.0);
        double2 uqp = -s * conj(e), uqq = c * conj(e);
        for (int k = 0; k < n; ++k) {  // A <- A U
          double2 x = A[k * n + p], y = A[k * n + q];
          A[k * n + p] = x * upp + y * uqp;
          A[k * n + q] = x * upq + y * uqq;
        }
        for (int k = 0; k < n; ++k) {  // A <- U^H A
          double2 x = A[p * n + k], y = A[q * n + k];
          A[p * n + k] = conj(upp) * x + conj(uqp) * y;
          A[q * n + k] = conj(upq) * x + conj(uqq) * y;
        }
        A[p * n + q] = mkc(0.0, 0.0);
        A[q * n + p] = mkc(0.0, 0.0);
        A[p * n + p].y = 0;
        A[q * n + q].y = 0;
        for (int k = 0; k < n; ++k) {  // V <- V U
          double2 x = V[k * n + p], y = V[k * n + q];
          V[k * n + p] = x * upp + y * uqp;
          V[k * n + q] = x * upq + y * uqq;
        }
      }
    }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i * n + i].x;
  // ascending order (selection sort keeps it deterministic)
  for (int i = 0; i < n; ++i) {
    int m = i;
    for (int j = i + 1; j < n; ++j)
      if (w[j] < w[m]) m = j;
    if (m != i) {
      double t = w[i]; w[i] = w[m]; w[m] = t;
      for (int k = 0; k < n; ++k) { double2 x = V[k * n + i]; V[k * n + i] = V[k * n + m]; V[k * n + m] = x; }
    }
  }
}

// ------------------------------------------------------------------ warp --
// Shared-memory matrices: row-major with leading dimension ld, lane = row.

// out = A * Bre (Bre real n x n, row-major ld_b), scaled; out may not alias A
template <typename R>
__device__ __forceinline__ void wmm_cr(cx<R>* out, const cx<R>* A, const double* Bre, int n, int ld,
                                       R scale) {
  const int i = threadIdx.x & 31;
  if (i < n) {
    for (int j = 0; j < n; ++j) {
      cx<R> acc = cmk<R>(0, 0);
      for (int k = 0; k < n; ++k) acc += (R)Bre[k * n + j] * A[i * ld + k];
      out[i * ld + j] = scale * acc;
    }
  }
  __syncwarp();
}

// out += scale * Are * B (Are real)
template <typename R>
__device__ __forceinline__ void wmm_rc_acc(cx<R>* out, const double* Are, const cx<R>* B, int n, int ld,
                                           R scale) {
  const int i = threadIdx.x & 31;
  if (i < n) {
    for (int j = 0; j < n; ++j) {
      cx<R> acc = cmk<R>(0, 0);
      for (int k = 0; k < n; ++k) acc += (R)Are[i * n + k] * B[k * ld + j];
      out[i * ld + j] += scale * acc;
    }
  }
  __syncwarp();
}

// Solve A X = B in place (A destroyed, B <- X), n x n with nrhs = n.
// Returns false on a zero pivot.
template <typename R>
__device__ bool wsolve(cx<R>* A, cx<R>* B, int n, int ld) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int k = 0; k < n; ++k) {
    R v = (lane >= k && lane < n) ? cabs1(A[lane * ld + k]) : (R)-1;
    int idx = lane;
    for (int off = 16; off > 0; off >>= 1) {
      R ov = __shfl_down_sync(0xffffffffu, v, off);
      int oi = __shfl_down_sync(0xffffffffu, idx, off);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    const int p = __shfl_sync(0xffffffffu, idx, 0);
    const R pv = __shfl_sync(0xffffffffu, v, 0);
    if (!(pv > 0)) { ok = false; }
    if (p != k) {
      for (int j = lane; j < n; j += 32) {
        cx<R> t = A[k * ld + j]; A[k * ld + j] = A[p * ld + j]; A[p * ld + j] = t;
        t = B[k * ld + j]; B[k * ld + j] = B[p * ld + j]; B[p * ld + j] = t;
      }
    }
    __syncwarp();
    if (lane > k && lane < n && ok) {
      cx<R> l = cdiv(A[lane * ld + k], A[k * ld + k]);
      A[lane * ld + k] = l;
      for (int j = k + 1; j < n; ++j) A[lane * ld + j] -= l * A[k * ld + j];
      for (int j = 0; j < n; ++j) B[lane * ld + j] -= l * B[k * ld + j];
    }
    __syncwarp();
  }
  if (!ok) return false;
  for (int k = n - 1; k >= 0; --k) {
    for (int j = lane; j < n; j += 32) B[k * ld + j] = cdiv(B[k * ld + j], A[k * ld + k]);
    __syncwarp();
    if (lane < k) {
      cx<R> a = A[lane * ld + k];
      for (int j = 0; j < n; ++j) B[lane * ld + j] -= a * B[k * ld + j];
    }
    __syncwarp();
  }
  return true;
}

}  // namespace pgb
