// Kernels and stage drivers of the GB300 FLEX engine (see flex.cuh).
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>

#include "flex.cuh"
#include "linalg.cuh"

namespace pgb {

namespace {
constexpr double kPi = 3.141592653589793238462643383279;
constexpr double kThresh = 1.0e-9;  // small-part zeroing of chi0 and Sigma (fchi.f90:483-506)

__host__ __device__ __forceinline__ long long fidx(long long k, long long j, long long a, long long b,
                                                   long long Nk, long long Nw, long long n) {
  return k + Nk * (j + Nw * (a + n * b));
}

template <typename T> __device__ __forceinline__ T thresh(T v) {
  if (fabs((double)v.x) < kThresh) v.x = 0;
  if (fabs((double)v.y) < kThresh) v.y = 0;
  return v;
}

// Device error flags, one slot per context: a kernel that finds a singular
// matrix or an unconverged eigenvalue iteration writes its code to the slot
// its launch was given (ctx().err), and the host reads it after the stage
__device__ int g_err_slots[kErrSlots];

}  // namespace

int* err_slot_address(int slot) {
  void* p = nullptr;
  PGB_CUDA(cudaGetSymbolAddress(&p, g_err_slots));
  return static_cast<int*>(p) + slot;
}

namespace {

// every launch of a flag-raising kernel follows a reset_err on its context
void reset_err() {
  PGB_CHECK(ctx().err != nullptr, "the engine context is not set up (no device error flag)");
  PGB_CUDA(cudaMemsetAsync(ctx().err, 0, sizeof(int), ctx().stream));
}
int fetch_err() {
  int e = 0;
  PGB_CUDA(cudaMemcpyAsync(&e, ctx().err, sizeof(int), cudaMemcpyDeviceToHost, ctx().stream));
  sync();
  return e;
}

inline void count_launch(const char* what) {
  launch_check(what);
  ctx().kernel_launches++;
}

inline unsigned grid_1d(long long n, int threads, long long cap = 1LL << 30) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}
}  // namespace

void log(const char* fmt, ...) {
  if (!ctx().verbose) return;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stdout, fmt, ap);
  va_end(ap);
  fflush(stdout);
}

// =============================================================== geometry ==
void build_geom(Geom& g, const int64_t* kmap, const int64_t* invk, int64_t Nx, int64_t Ny, int64_t Nz,
                int64_t Nk, int64_t Nw, int64_t Norb, int64_t Nchi) {
  PGB_CHECK(Nx > 0 && Ny > 0 && Nz > 0 && Nk > 0 && Nw > 0 && Norb > 0 && Nchi > 0,
            "non-positive mesh or orbital dimension");
  PGB_CHECK(Norb <= kMaxOrb, "Norb above the engine limit of 8 orbitals");
  PGB_CHECK(Nchi <= kMaxChi, "Nchi above the engine limit of 32 orbital pairs");
  g.Nx = (int)Nx; g.Ny = (int)Ny; g.Nz = (int)Nz; g.Nw = (int)Nw; g.Nk = (int)Nk;
  g.Norb = (int)Norb; g.Nchi = (int)Nchi;
  for (int a = 0; a < kMaxOrb; ++a) {
    g.spin.inv[a] = a;
    g.spin.sgn[a] = 1;
  }
  g.spin.on = 0;
  g.Nkall = Nx * Ny * Nz;
  g.M = 2 * Nw;
  g.P = g.Nkall * g.M;
  g.K = Nk * Nw;
  g.h_grid_irr.assign(g.Nkall, -1);
  g.h_grid_flag.assign(g.Nkall, 0);
  g.h_irr_grid.assign(Nk, -1);
  g.h_kweight.assign(Nk, 0.0);
  g.h_full_of_grid.assign(g.Nkall, -1);
  g.h_kmap.assign(kmap, kmap + 3 * g.Nkall);
  for (long long i = 0; i < g.Nkall; ++i) {
    const int64_t x = kmap[3 * i], y = kmap[3 * i + 1], z = kmap[3 * i + 2];
    PGB_CHECK(x >= 0 && x < Nx && y >= 0 && y < Ny && z >= 0 && z < Nz, "kmap entry outside the mesh");
    const long long gi = x + Nx * (y + Ny * z);
    PGB_CHECK(g.h_grid_irr[gi] < 0, "kmap maps two k points onto one mesh cell");
    const int64_t k = invk[3 * i] - 1, fl = invk[3 * i + 1];
    PGB_CHECK(k >= 0 && k < Nk, "invk(1,:) outside [1,Nk]");
    PGB_CHECK(fl == 0 || fl == 1, "invk(2,:) must be 0 or 1");
    g.h_grid_irr[gi] = (int)k;
    g.h_grid_flag[gi] = (int)fl;
    g.h_full_of_grid[gi] = (int)i;
    g.h_kweight[k] += 1.0;
    if (fl == 0) {
      PGB_CHECK(g.h_irr_grid[k] < 0, "an irreducible k point has two direct images");
      g.h_irr_grid[k] = (int)gi;
    }
  }
  for (long long k = 0; k < Nk; ++k)
    PGB_CHECK(g.h_irr_grid[k] >= 0, "an irreducible k point has no direct image in kmap/invk");
  g.grid_irr.alloc(g.Nkall);
  g.grid_irr.upload(g.h_grid_irr.data(), g.Nkall);
  g.grid_flag.alloc(g.Nkall);
  g.grid_flag.upload(g.h_grid_flag.data(), g.Nkall);
  g.irr_grid.alloc(Nk);
  g.irr_grid.upload(g.h_irr_grid.data(), Nk);
  g.kweight.alloc(Nk);
  g.kweight.upload(g.h_kweight.data(), Nk);
}

void build_pairs(Pairs& p, const int64_t* olist, int Norb, int Nchi, const int32_t* irr_chi,
                 const int32_t* chi_map) {
  p.Norb = Norb;
  p.Nchi = Nchi;
  p.o1.resize(Nchi);
  p.o2.resize(Nchi);
  for (int l = 0; l < Nchi; ++l) {
    p.o1[l] = (int)olist[l] - 1;
    p.o2[l] = (int)olist[Nchi + l] - 1;
    PGB_CHECK(p.o1[l] >= 0 && p.o1[l] < Norb && p.o2[l] >= 0 && p.o2[l] < Norb,
              "olist entry outside [1,Norb]");
  }
  // exchange-symmetry map chi_1234 = chi*_4321 (fchi.f90:421-481)
  std::vector<int> cm_m(Nchi * Nchi, -1), cm_l(Nchi * Nchi, -1);
  std::vector<std::pair<int, int>> irr;  // (l, m)
  if (chi_map && irr_chi) {
    for (int l = 0; l < Nchi; ++l)
      for (int m = 0; m < Nchi; ++m) {
        cm_m[m + Nchi * l] = chi_map[m + Nchi * l] - 1;
        cm_l[m + Nchi * l] = chi_map[m + Nchi * (l + Nchi)] - 1;
      }
    const int nirr = Nchi * (Nchi + 1) / 2;
    for (int it = 0; it < nirr; ++it) {
      const int l = irr_chi[it] - 1, m = irr_chi[it + nirr] - 1;
      if (l < 0 || m < 0) continue;
      PGB_CHECK(l < Nchi && m < Nchi, "irr_chi entry outside [1,Nchi]");
      irr.push_back({l, m});
    }
  } else {
    std::vector<char> is_irr(Nchi * Nchi, 0);
    for (int l1 = 0; l1 < Nchi; ++l1)
      for (int m1 = 0; m1 < Nchi; ++m1) {
        bool done = false;
        for (int l2 = 0; l2 < Nchi && !done; ++l2)
          for (int m2 = 0; m2 < Nchi; ++m2) {
            if (p.o1[l1] == p.o2[m2] && p.o2[l1] == p.o1[m2] && p.o1[m1] == p.o2[l2] &&
                p.o2[m1] == p.o1[l2]) {
              cm_m[m1 + Nchi * l1] = m2;
              cm_l[m1 + Nchi * l1] = l2;
              if (!is_irr[m2 + Nchi * l2]) is_irr[m1 + Nchi * l1] = 1;
              done = true;
              break;
            }
          }
      }
    for (int l1 = 0; l1 < Nchi; ++l1)
      for (int m1 = 0; m1 < Nchi; ++m1)
        if (is_irr[m1 + Nchi * l1]) irr.push_back({l1, m1});
  }
  p.chi.clear();
  for (auto& lm : irr) {
    ChiPair c{};
    c.l = lm.first;
    c.m = lm.second;
    c.m2 = cm_m[c.m + Nchi * c.l];
    c.l2 = cm_l[c.m + Nchi * c.l];
    PGB_CHECK(c.m2 >= 0 && c.l2 >= 0, "orbital pair without exchange partner in olist");
    c.self = (c.m2 == c.m && c.l2 == c.l);
    c.e13 = p.o1[c.l] + Norb * p.o1[c.m];
    c.e42 = p.o2[c.m] + Norb * p.o2[c.l];
    c.J = make_double2(0, 0);
    p.chi.push_back(c);
  }
  p.sigma.assign(Norb * Norb, {});
  p.delta.assign(Norb * Norb, {});
  for (int l = 0; l < Nchi; ++l)
    for (int m = 0; m < Nchi; ++m) {
      p.sigma[p.o1[m] + Norb * p.o1[l]].push_back({m, l, p.o2[m] + Norb * p.o2[l]});
      if (p.o1[l] >= p.o2[m]) p.delta[p.o1[l] + Norb * p.o2[m]].push_back({m, l, p.o2[l] + Norb * p.o1[m]});
    }
}

void build_pairs_soc(Pairs& p, Geom& g, const int64_t* olist, int Norb, int Nchi, const int64_t* invs,
                     const int64_t* slist) {
  PGB_CHECK(Norb <= kMaxOrb, "Norb above the engine limit of 8 orbitals");
  for (int a = 0; a < Norb; ++a) {
    PGB_CHECK(invs[a] >= 1 && invs[a] <= Norb, "invs entry outside [1,Norb]");
    PGB_CHECK(slist[a] == 1 || slist[a] == -1, "slist entries must be +1 or -1");
    g.spin.inv[a] = (int)invs[a] - 1;
    g.spin.sgn[a] = (int)slist[a];
  }
  for (int a = 0; a < Norb; ++a)
    PGB_CHECK(g.spin.inv[g.spin.inv[a]] == a, "invs is not an involution");
  g.spin.on = 1;
  std::vector<int> o1(Nchi), o2(Nchi);
  for (int l = 0; l < Nchi; ++l) {
    o1[l] = (int)olist[l] - 1;
    o2[l] = (int)olist[Nchi + l] - 1;
    PGB_CHECK(o1[l] >= 0 && o1[l] < Norb && o2[l] >= 0 && o2[l] < Norb, "olist entry outside [1,Norb]");
  }
  // chi_1234 = sgn chi*_{-4,-3,-2,-1}: pair (m1,l1) maps to (m2,l2) with
  // (o1 l1, o2 l1, o1 m1, o2 m1) = (inv o2 m2, inv o1 m2, inv o2 l2, inv o1 l2)
  const int* inv = g.spin.inv;
  std::vector<int32_t> cmap(2 * (size_t)Nchi * Nchi, 0);
  const int nirr = Nchi * (Nchi + 1) / 2;
  std::vector<int32_t> irr(2 * (size_t)nirr, 0);
  std::vector<char> is_irr((size_t)Nchi * Nchi, 0);
  for (int l1 = 0; l1 < Nchi; ++l1)
    for (int m1 = 0; m1 < Nchi; ++m1) {
      bool done = false;
      for (int l2 = 0; l2 < Nchi && !done; ++l2)
        for (int m2 = 0; m2 < Nchi; ++m2) {
          if (o1[l1] == inv[o2[m2]] && o2[l1] == inv[o1[m2]] && o1[m1] == inv[o2[l2]] && o2[m1] == inv[o1[l2]]) {
            cmap[m1 + (size_t)Nchi * l1] = m2 + 1;
            cmap[m1 + (size_t)Nchi * (l1 + Nchi)] = l2 + 1;
            if (!is_irr[m2 + (size_t)Nchi * l2]) is_irr[m1 + (size_t)Nchi * l1] = 1;
            done = true;
            break;
          }
        }
    }
  int it = 0;
  for (int l1 = 0; l1 < Nchi; ++l1)
    for (int m1 = 0; m1 < Nchi; ++m1)
      if (is_irr[m1 + (size_t)Nchi * l1]) {
        PGB_CHECK(it < nirr, "more irreducible spin-orbit pairs than Nchi(Nchi+1)/2");
        irr[it] = l1 + 1;
        irr[it + nirr] = m1 + 1;
        ++it;
      }
  build_pairs(p, olist, Norb, Nchi, irr.data(), cmap.data());
  for (auto& c : p.chi) {
    const int sg = g.spin.sgn[o1[c.l]] * g.spin.sgn[o2[c.l]] * g.spin.sgn[o1[c.m]] * g.spin.sgn[o2[c.m]];
    c.pneg = sg < 0 ? 1 : 0;
  }
}

// =============================================================== green ==
// Band projectors C(k)_{ml,n} = U_mn(k) conj(U_ln(k)) at cf[((k No + l) No + m) No + n]
// (element e = m + No l), used by G0 and the tail's tau reference; they do
// not depend on the frequency or the imaginary time
__global__ void k_band_proj(double2* cf, const double2* uni, int Nk, int No) {
  const long long N = (long long)Nk * No * No * No;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(idx % No);
    const long long r = idx / No;
    const int e = (int)(r % (No * No));
    const int k = (int)(r / (No * No));
    const int m = e % No, l = e / No;
    const double2* U = uni + (long long)No * No * k;
    cf[idx] = U[m + No * n] * conj(U[l + No * n]);
  }
}

void band_projectors(double2* cf, const double2* uni, int Nk, int Norb) {
  const long long N = (long long)Nk * Norb * Norb * Norb;
  k_band_proj<<<grid_1d(N, 256, 65536), 256, 0, ctx().stream>>>(cf, uni, Nk, Norb);
  count_launch("band_proj");
}

// G0_ml(k, i w_j) = sum_n C(k)_{ml,n} / (i w_j + mu - e_n(k)) (fself.f90:1-41),
// one reciprocal per band and (k, j)
__global__ void k_green0(double2* G, const double* eig, const double2* cf, double mu, double temp,
                         int Nk, int Nw, int No) {
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk), j = (int)(idx / Nk);
    const double2 iw = mkc(mu, (2.0 * j + 1.0) * kPi * temp);
    double2 den[kMaxOrb];
    for (int n = 0; n < No; ++n) den[n] = crecip(iw - mkc(eig[n + (long long)No * k], 0.0));
    const double2* C = cf + (long long)No * No * No * k;
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m) {
        const double2* c = C + (long long)(m + No * l) * No;
        double2 acc = mkc(0.0, 0.0);
        for (int n = 0; n < No; ++n) acc += c[n] * den[n];
        G[fidx(k, j, m, l, Nk, Nw, No)] = acc;
      }
  }
}

void green0(double2* G, const double* eig, const double2* uni, double mu, double temp, int Nk, int Nw,
            int Norb) {
  const long long K = (long long)Nk * Nw;
  DBuf<double2> cf((size_t)Nk * Norb * Norb * Norb);
  band_projectors(cf.p, uni, Nk, Norb);
  k_green0<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(G, eig, cf.p, mu, temp, Nk, Nw, Norb);
  count_launch("green0");
}

__global__ void k_dyson(double2* G, const double2* sig, const double2* hamk, double mu, double temp,
                        int Nk, int Nw, int No, int invert, int* err) {
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk), j = (int)(idx / Nk);
    const double2 iw = mkc(mu, (2.0 * j + 1.0) * kPi * temp);
    double2 A[kMaxOrb * kMaxOrb];
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m) {
        double2 v = -(hamk[m + No * (l + (long long)No * k)] + sig[fidx(k, j, m, l, Nk, Nw, No)]);
        if (l == m) v += iw;
        A[m * No + l] = v;
      }
    if (invert && !inv_small(A, No)) atomicExch(err, 1);
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m) G[fidx(k, j, m, l, Nk, Nw, No)] = A[m * No + l];
  }
}

bool dyson(double2* G, const double2* sig, const double2* hamk, double mu, double temp, int Nk, int Nw,
           int Norb) {
  reset_err();
  const long long K = (long long)Nk * Nw;
  k_dyson<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(G, sig, hamk, mu, temp, Nk, Nw, Norb, 1, ctx().err);
  count_launch("dyson");
  return fetch_err() == 0;
}

void green_inv_only(double2* G, const double2* sig, const double2* hamk, double mu, double temp, int Nk,
                    int Nw, int Norb) {
  const long long K = (long long)Nk * Nw;
  k_dyson<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(G, sig, hamk, mu, temp, Nk, Nw, Norb, 0, ctx().err);
  count_launch("green_inv");
}

__global__ void k_invert_blocks(double2* G, long long nmat, int No, long long smat, long long sel, int* err) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nmat;
       t += (long long)gridDim.x * blockDim.x) {
    double2 A[kMaxOrb * kMaxOrb];
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m) A[m * No + l] = G[t * smat + sel * (m + No * l)];
    if (!inv_small(A, No)) atomicExch(err, 1);
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m) G[t * smat + sel * (m + No * l)] = A[m * No + l];
  }
}

bool invert_blocks(double2* G, long long nmat, int Norb, long long stride_mat, long long stride_el) {
  reset_err();
  k_invert_blocks<<<grid_1d(nmat, 128, 65536), 128, 0, ctx().stream>>>(G, nmat, Norb, stride_mat,
                                                                         stride_el, ctx().err);
  count_launch("invert_blocks");
  return fetch_err() == 0;
}

// ====================================================== mesh x time grids ==
// Kernels over a padded array of P = Nkall x M points (mesh point r fastest)
// give each thread one mesh point r and up to kTauChunk consecutive slices t
// (blocks of 256 threads: the mesh in blocks, then the slices in chunks).
// The mesh index is split once per thread in 32-bit arithmetic, and the
// per-point tables (grid_irr, grid_flag, reversed indices) are read once;
// a grid-stride loop over P would split every element's index with 64-bit
// divisions, which on GB300 cost far more than the element's own loads.
constexpr int kTauChunk = 8;

dim3 mesh_tau_grid(long long Nkall, long long M, unsigned ny, int chunk = kTauChunk) {
  const long long nrb = (Nkall + 255) / 256, nch = (M + chunk - 1) / chunk;
  return dim3((unsigned)(nrb * nch), ny);
}

struct MeshTau {
  int r, t0, t1;
};
__device__ __forceinline__ bool mesh_tau(long long Nkall, long long M, MeshTau& q, int chunk = kTauChunk) {
  const unsigned nrb = (unsigned)((Nkall + 255) / 256);
  const unsigned rb = blockIdx.x % nrb, tc = blockIdx.x / nrb;
  q.r = (int)(rb * 256u + threadIdx.x);
  q.t0 = (int)tc * chunk;
  q.t1 = min((int)M, q.t0 + chunk);
  return q.r < Nkall;
}

// ========================================================== padded grids ==
// Full-grid padded Green function of element e=(a,b) (fchi.f90:563-583):
// slot n<Nw: G_ab(k,iw_n) (at -k: G_ba), slot 2Nw-1-j: conj G_ba(k,iw_j)
// (at -k: conj G_ab).
template <typename R>
__global__ void k_pad_green(cx<R>* out, const double2* G, const int* elems, const int* grid_irr,
                            const int* grid_flag, long long Nkall, int Nk, int Nw, int No, long long P,
                            SpinMap sm) {
  const int e = elems[blockIdx.y];
  const int a = e % No, b = e / No;
  const int ia = sm.inv[a], ib = sm.inv[b];
  const double sg = (double)(sm.sgn[a] * sm.sgn[b]);
  cx<R>* o = out + (long long)blockIdx.y * P;
  MeshTau q;
  if (!mesh_tau(Nkall, 2LL * Nw, q)) return;
  const long long gi = q.r;
  const int k = grid_irr[gi], fl = grid_flag[gi];
  for (int n = q.t0; n < q.t1; ++n) {
    const long long idx = gi + Nkall * n;
    double2 v;
    if (n < Nw) {
      v = fl ? sg * G[fidx(k, n, ib, ia, Nk, Nw, No)] : G[fidx(k, n, a, b, Nk, Nw, No)];
    } else {
      const int j = 2 * Nw - 1 - n;
      v = fl ? sg * conj(G[fidx(k, j, ia, ib, Nk, Nw, No)]) : conj(G[fidx(k, j, b, a, Nk, Nw, No)]);
    }
    o[idx] = cmk<R>((R)v.x, (R)v.y);
  }
}

// Padded bosonic array of pair (m,l) (fself.f90:201-223, feliash.f90:538-560):
// slots 0..Nw-1 = nu_0..nu_{Nw-1} (at -q the transposed pair), slot Nw = the
// static value, slot 2Nw-j = conj V_lm(nu_j) (at -q conj V_ml).
struct BosonTerm {
  int m, l;
  double stat;
};
template <typename R>
__global__ void k_pad_boson(cx<R>* out, const cx<R>* V, const BosonTerm* terms, const int* grid_irr,
                            const int* grid_flag, long long Nkall, int Nk, int Nw, int Nchi, long long P) {
  const BosonTerm t = terms[blockIdx.y];
  cx<R>* o = out + (long long)blockIdx.y * P;
  __shared__ R s_stat;  // converted once per block (see k_chi0_scatter)
  if (threadIdx.x == 0) s_stat = (R)t.stat;
  __syncthreads();
  const R stat = s_stat;
  MeshTau q;
  if (!mesh_tau(Nkall, 2LL * Nw, q)) return;
  const long long gi = q.r;
  const int k = grid_irr[gi], fl = grid_flag[gi];
  for (int n = q.t0; n < q.t1; ++n) {
    const long long idx = gi + Nkall * n;
    cx<R> v;
    if (n < Nw) {
      v = fl ? V[fidx(k, n, t.l, t.m, Nk, Nw, Nchi)] : V[fidx(k, n, t.m, t.l, Nk, Nw, Nchi)];
    } else if (n == Nw) {
      v = cmk<R>(stat, (R)0);
    } else {
      const int j = 2 * Nw - n;
      v = conj(fl ? V[fidx(k, j, t.m, t.l, Nk, Nw, Nchi)] : V[fidx(k, j, t.l, t.m, Nk, Nw, Nchi)]);
    }
    o[idx] = v;
  }
}

// Padded anomalous function of element (a,b) with the parity rules of
// mkdelta_nsoc (feliash.f90:561-578).
template <typename R>
__global__ void k_pad_anomalous(cx<R>* out, const double2* F, const int* grid_irr, const int* grid_flag,
                                long long Nkall, int Nk, int Nw, int No, long long P, const double* prt,
                                double sgn, double dprt) {
  const int e = blockIdx.y;
  const int a = e % No, b = e / No;
  const double pp = prt[a] * prt[b];
  cx<R>* o = out + (long long)e * P;
  MeshTau q;
  if (!mesh_tau(Nkall, 2LL * Nw, q)) return;
  const long long gi = q.r;
  const int k = grid_irr[gi], fl = grid_flag[gi];
  for (int n = q.t0; n < q.t1; ++n) {
    const long long idx = gi + Nkall * n;
    double2 v;
    if (n < Nw) {
      v = F[fidx(k, n, a, b, Nk, Nw, No)];
      if (fl) v = (pp * dprt) * v;
    } else {
      const int j = 2 * Nw - 1 - n;
      if (!fl) v = (sgn * dprt * pp) * conj(F[fidx(k, j, a, b, Nk, Nw, No)]);
      else v = sgn * F[fidx(k, j, b, a, Nk, Nw, No)];
    }
    o[idx] = cmk<R>((R)v.x, (R)v.y);
  }
}

// The same padding from an anomalous function already in the bulk type
// (the double-float F of the mixed Eliashberg stage).  The parity factors
// are signs (prt = +-1, checked by the caller), applied as sign changes.
template <typename R>
__global__ void k_pad_anomalous_bulk(cx<R>* out, const cx<R>* F, const int* grid_irr, const int* grid_flag,
                                     long long Nkall, int Nk, int Nw, int No, long long P, const double* prt,
                                     double sgn, double dprt) {
  const int e = blockIdx.y;
  const int a = e % No, b = e / No;
  const double pp = prt[a] * prt[b];
  const bool neg_fl = pp * dprt < 0, neg_mirror = sgn * dprt * pp < 0, neg_sgn = sgn < 0;
  cx<R>* o = out + (long long)e * P;
  MeshTau q;
  if (!mesh_tau(Nkall, 2LL * Nw, q)) return;
  const long long gi = q.r;
  const int k = grid_irr[gi], fl = grid_flag[gi];
  for (int n = q.t0; n < q.t1; ++n) {
    const long long idx = gi + Nkall * n;
    cx<R> v;
    if (n < Nw) {
      v = F[fidx(k, n, a, b, Nk, Nw, No)];
      if (fl && neg_fl) v = -v;
    } else {
      const int j = 2 * Nw - 1 - n;
      if (!fl) {
        v = conj(F[fidx(k, j, a, b, Nk, Nw, No)]);
        if (neg_mirror) v = -v;
      } else {
        v = F[fidx(k, j, b, a, Nk, Nw, No)];
        if (neg_sgn) v = -v;
      }
    }
    o[idx] = v;
  }
}

template <typename R>
void pad_green_all(const Geom& g, const double2* G, cx<R>* out) {
  const int No2 = g.Norb * g.Norb;
  std::vector<int> h(No2);
  for (int e = 0; e < No2; ++e) h[e] = e;
  DBuf<int> d(No2);
  d.upload(h.data(), No2);
  k_pad_green<R><<<mesh_tau_grid(g.Nkall, g.M, No2), 256, 0, ctx().stream>>>(out, G, d.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk,
                                                  g.Nw, g.Norb, g.P, g.spin);
  count_launch("pad_green");
}

// ================================================================== chi0 ==
// One backward transform of chi0: pair (l,m) written at element (m,l) and its
// exchange partner (m2,l2).  If has_d, the same transform also yields the
// swapped pair (m,l): chi_ml(q,nu) = conj chi_lm(q,-nu) holds term by term
// (padding, product, analytic tau reference; the sawtooth coefficient is its
// own dJ), so the swapped pair is read from the negative frequencies and
// written at (dm,dl) and its partner (dm2,dl2).
struct ChiDev {
  int m, l, m2, l2, e13, e42, self, has_d;
  double2 J;
  int dm, dl, dm2, dl2;
  double2 dJ;
  int pneg;  // partner = -conj (spin-orbit exchange sign)
};

template <typename R>
__global__ void k_chi0_product(cx<R>* out, const cx<R>* F, const cx<R>* F0, const cx<R>* A,
                               const cx<R>* B, const ChiDev* pairs, long long P, int Nx, int Ny, int Nz,
                               int M, const int* rx, const int* ry, const int* rz, const int* rt,
                               const int* lt, R sc, R sr) {
  const ChiDev pr = pairs[blockIdx.y];
  const cx<R>* a13 = F + (long long)pr.e13 * P;
  const cx<R>* b42 = F + (long long)pr.e42 * P;
  cx<R>* o = out + (long long)blockIdx.y * P;
  const int Nxy = Nx * Ny, Nkall = Nxy * Nz;
  MeshTau q;
  if (!mesh_tau(Nkall, M, q)) return;
  const int r = q.r;
  const int x = r % Nx, y = (r / Nx) % Ny, z = r / Nxy;
  const long long rr = rx[x] + (long long)Nx * (ry[y] + (long long)Ny * rz[z]);
  for (int t = q.t0; t < q.t1; ++t) {
    const long long idx = r + (long long)Nkall * t;
    const long long ir = rr + (long long)Nkall * rt[t];
    cx<R> v = -(a13[idx] * b42[ir]);
    if (F0) {
      // The reference conjugates a self-partner pair after each of its three
      // accumulations (fchi.f90:610, 845-846), which leaves conj(conv[G] + ref)
      // - conv[G0]; conj(conv[G0]) enters here as the transform of
      // conj(P0(-r,-t)) so that one backward FFT and a final conj give it.
      if (pr.self) v += conj(F0[(long long)pr.e13 * P + ir] * F0[(long long)pr.e42 * P + idx]);
      else v += F0[(long long)pr.e13 * P + idx] * F0[(long long)pr.e42 * P + ir];
    }
    v = sc * v;
    if (A) {
      const long long s = lt[t];
      v -= sr * (A[(long long)pr.e13 * P + r + Nkall * s] * B[(long long)pr.e42 * P + rr + Nkall * s]);
    }
    o[idx] = v;
  }
}

template <typename R>
__global__ void k_chi0_scatter(cx<R>* chi, const cx<R>* tmp, const ChiDev* pairs, const int* irr_grid,
                               const cx<R>* sawc, long long Nkall, int Nk, int Nw, int Nchi, long long P) {
  const ChiDev pr = pairs[blockIdx.y];
  const cx<R>* t = tmp + (long long)blockIdx.y * P;
  // the pair's tau-jump coefficients, converted once per block: a double ->
  // R conversion runs on the FP64 pipe (1/64 of the FP32 rate on GB300)
  __shared__ cx<R> sJ[2];
  if (threadIdx.x == 0) {
    sJ[0] = cmk<R>((R)pr.J.x, (R)pr.J.y);
    sJ[1] = cmk<R>((R)pr.dJ.x, (R)pr.dJ.y);
  }
  __syncthreads();
  const cx<R> J = sJ[0], dJ = sJ[1];
  MeshTau q;  // here: one irreducible k, a chunk of frequencies j
  if (!mesh_tau(Nk, Nw, q)) return;
  const int k = q.r;
  const long long gk = irr_grid[k];
  for (int j = q.t0; j < q.t1; ++j) {
    cx<R> v = t[gk + Nkall * j];
    if (sawc) v += J * sawc[j];
    if (pr.self) v = pr.pneg ? -conj(v) : conj(v);
    if (abs_below(v.x, kThresh)) v.x = 0;
    if (abs_below(v.y, kThresh)) v.y = 0;
    chi[fidx(k, j, pr.m, pr.l, Nk, Nw, Nchi)] = v;
    if (!pr.self) chi[fidx(k, j, pr.m2, pr.l2, Nk, Nw, Nchi)] = pr.pneg ? -conj(v) : conj(v);
    if (pr.has_d) {
      const long long M = 2LL * Nw;
      cx<R> d = conj(t[gk + Nkall * ((M - j) % M)]);
      if (sawc) d += dJ * sawc[j];
      if (abs_below(d.x, kThresh)) d.x = 0;
      if (abs_below(d.y, kThresh)) d.y = 0;
      chi[fidx(k, j, pr.dm, pr.dl, Nk, Nw, Nchi)] = d;
      chi[fidx(k, j, pr.dm2, pr.dl2, Nk, Nw, Nchi)] = conj(d);
    }
  }
}

// tau kernels of the analytic reference bubble (fchi.f90:703-729), laid out
// [(s*Norb + n)*Nk + k]
template <typename T>
__global__ void k_gpm(T* gp, T* gm, double* ff, const double* eig, double mu, double temp,
                      int Nk, int No, int M) {
  const double beta = 1.0 / temp, dtau = beta / M;
  const int Nkn = Nk * No;
  MeshTau mt;  // here: one (n, k) pair, a chunk of tau slices s
  if (!mesh_tau(Nkn, M, mt)) return;
  const int k = mt.r % Nk, n = mt.r / Nk;
  const double xi = eig[n + (long long)No * k] - mu;
  for (int s = mt.t0; s < mt.t1; ++s) {
    const long long idx = mt.r + (long long)Nkn * s;
    const double tau = s * dtau;
    if constexpr (std::is_same<T, float>::value) {
      // FP32 kernels for an FP32 chi0: the exponents in FP64, the
      // exponentials in FP32 (their FP64 forms run at 1/64 of the rate)
      const float e = expf((float)(-beta * fabs(xi)));
      const float rd = 1.0f / (1.0f + e);
      const float lo = expf((float)(-fabs(xi) * tau)), hi = expf((float)(-fabs(xi) * (beta - tau)));
      gp[idx] = xi >= 0 ? -lo * rd : -hi * rd;
      gm[idx] = xi >= 0 ? hi * rd : lo * rd;
      if (s == 0) {
        const double d = 1.0 + exp(-beta * fabs(xi));
        ff[n + (long long)No * k] = xi >= 0 ? exp(-beta * xi) / d : 1.0 / d;
      }
      continue;
    }
    double p, q;
    if (xi >= 0) {
      const double d = 1.0 + exp(-beta * xi);
      p = -exp(-xi * tau) / d;
      q = exp(-xi * (beta - tau)) / d;
      if (s == 0) ff[n + (long long)No * k] = exp(-beta * xi) / d;
    } else {
      const double d = 1.0 + exp(beta * xi);
      p = -exp(xi * (beta - tau)) / d;
      q = exp(xi * tau) / d;
      if (s == 0) ff[n + (long long)No * k] = 1.0 / d;
    }
    gp[idx] = (T)p;
    gm[idx] = (T)q;
  }
}

// A_ab(g,s) = sum_n U_an U*_bn gp (conjugated at -k), same for B with gm, from
// the band projectors; in FP32 for an FP32 chi0, in FP64 otherwise (T)
template <typename R, typename T>
__global__ void k_ref_tau(cx<R>* A, cx<R>* B, const T* gp, const T* gm, const cx<T>* cf,
                          const int* grid_irr, const int* grid_flag, long long Nkall, int Nk, int No,
                          int M, long long P) {
  const int e = blockIdx.y;
  MeshTau q;
  if (!mesh_tau(Nkall, M, q)) return;
  const long long gi = q.r;
  const int k = grid_irr[gi], fl = grid_flag[gi];
  const cx<T>* c = cf + ((long long)k * No * No + e) * No;
  for (int s = q.t0; s < q.t1; ++s) {
    const long long idx = gi + Nkall * s;
    cx<T> sa = cmk<T>((T)0, (T)0), sb = cmk<T>((T)0, (T)0);
    for (int n = 0; n < No; ++n) {
      const long long gidx = ((long long)s * No + n) * Nk + k;
      const cx<T> cn = c[n];
      sa += gp[gidx] * cn;
      sb += gm[gidx] * cn;
    }
    if (fl) {
      sa = conj(sa);
      sb = conj(sb);
    }
    A[(long long)e * P + idx] = cmk<R>((R)sa.x, (R)sa.y);
    B[(long long)e * P + idx] = cmk<R>((R)sb.x, (R)sb.y);
  }
}

// rhobar(m,l) = (1/Nkall) sum_full [rho(m,l,k) | rho(l,m,k) at -k] (fchi.f90:731-755)
__global__ void k_rhobar(double2* rhobar, const double2* uni, const double* ff, const int* grid_irr,
                         const int* grid_flag, long long Nkall, int No) {
  const int e = blockIdx.x;
  const int m = e % No, l = e / No;
  __shared__ double2 red[256];
  double2 acc = mkc(0.0, 0.0);
  for (long long gi = threadIdx.x; gi < Nkall; gi += blockDim.x) {
    const int k = grid_irr[gi], fl = grid_flag[gi];
    const int p = fl ? l : m, q = fl ? m : l;
    const double2* U = uni + (long long)No * No * k;
    double2 r = mkc(0.0, 0.0);
    for (int n = 0; n < No; ++n) r += (U[p + No * n] * conj(U[q + No * n])) * mkc(ff[n + (long long)No * k], 0.0);
    acc += r;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) rhobar[e] = (1.0 / (double)Nkall) * red[0];
}

// sawtooth correction: exact -1/(i nu) minus its rectangle-rule DFT (fchi.f90:757-772)
__global__ void k_sawc(double2* sawc, int Nw, int M, double temp) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Nw) return;
  const double dtau = 1.0 / temp / M;
  double2 v = mkc(0.0, 0.0);
  if (j > 0) v = mkc(0.0, 1.0 / (2.0 * kPi * j * temp));
  for (int s = 0; s < M; ++s) {
    double sn, cs;
    sincospi(2.0 * (double)(((long long)j * s) % M) / (double)M, &sn, &cs);
    const double w = dtau * (0.5 - (double)s / (double)M);
    v.x -= w * cs;
    v.y -= w * sn;
  }
  sawc[j] = v;
}

// PYRPA_GB_CHI0_SWAP=0 computes every exchange class with its own transform
bool chi0_swap_enabled() {
  const char* s = std::getenv("PYRPA_GB_CHI0_SWAP");
  return !(s && std::string(s) == "0");
}

template <typename R>
void chi0(const Geom& g, const Pairs& p, const double2* G, double temp, const TailRef* tail, cx<R>* chi) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, (int)g.M, (int)sizeof(cx<R>));
  const int No2 = g.Norb * g.Norb;
  DBuf<cx<R>> F((size_t)No2 * g.P);
  pad_green_all<R>(g, G, F.p);
  fft.forward<R>(F.p, No2, st);
  DBuf<cx<R>> F0, A, B, sawc;
  std::vector<ChiDev> hp(p.chi.size());
  for (size_t i = 0; i < p.chi.size(); ++i) {
    const ChiPair& c = p.chi[i];
    hp[i] = ChiDev{c.m, c.l, c.m2, c.l2, c.e13, c.e42, c.self, 0, make_double2(0, 0), 0, 0, 0, 0,
                   make_double2(0, 0), c.pneg};
  }
  // swapped partners: the relation chi_ml(q,nu) = conj chi_lm(q,-nu) is exact
  // for any G, while the exchange relation is imposed (the partner is written
  // as the conjugate of the class representative).  A class is therefore read
  // off p's transform only when its own representative is exactly W p = (m,l)
  // (derived[] = source); the other classes keep their transform.
  const int Nchi = g.Nchi;
  std::vector<int> cls((size_t)Nchi * Nchi, -1);  // element (m,l) -> index in hp
  for (size_t i = 0; i < hp.size(); ++i) {
    cls[hp[i].m + (size_t)Nchi * hp[i].l] = (int)i;
    cls[hp[i].m2 + (size_t)Nchi * hp[i].l2] = (int)i;
  }
  std::vector<int> derived(hp.size(), -1);  // source transform of a derived class
  if (chi0_swap_enabled() && !g.spin.on) {  // the derivation assumes unsigned partners
    for (size_t i = 0; i < hp.size(); ++i) {
      const ChiDev& c = hp[i];
      if (c.self || derived[i] >= 0 || c.has_d || c.l == c.m) continue;
      const int j = cls[c.l + (size_t)Nchi * c.m];  // class of W p (element (l,m))
      if (j < 0 || j == (int)i || hp[j].self || derived[j] >= 0 || hp[j].has_d) continue;
      if (hp[j].l != c.m || hp[j].m != c.l) continue;  // representative is E W p, not W p
      derived[j] = (int)i;
      ChiDev& s = hp[i];
      s.has_d = 1;
      s.dm = hp[j].m;  // W p = (l' = m, m' = l) is written at element (m', l') = (l, m)
      s.dl = hp[j].l;
      s.dm2 = hp[j].m2;
      s.dl2 = hp[j].l2;
    }
  }
  if (tail) {
    DBuf<double2> G0((size_t)g.K * No2);
    green0(G0.p, tail->eig, tail->uni, tail->mu, temp, g.Nk, g.Nw, g.Norb);
    F0.alloc((size_t)No2 * g.P);
    pad_green_all<R>(g, G0.p, F0.p);
    G0.release();
    fft.forward<R>(F0.p, No2, st);
    // the tau reference in FP32 for an FP32 chi0 (its rounding is below the
    // FP32 transforms'), in FP64 for the wider types
    using T = typename std::conditional<std::is_same<R, float>::value, float, double>::type;
    DBuf<T> gp((size_t)g.Nk * g.Norb * g.M), gm((size_t)g.Nk * g.Norb * g.M);
    DBuf<double> ff((size_t)g.Nk * g.Norb);
    k_gpm<T><<<mesh_tau_grid((long long)g.Nk * g.Norb, g.M, 1), 256, 0, st>>>(
        gp.p, gm.p, ff.p, tail->eig, tail->mu, temp, g.Nk, g.Norb, (int)g.M);
    count_launch("gpm");
    const size_t ncf = (size_t)g.Nk * g.Norb * No2;
    DBuf<double2> cf64(ncf);
    band_projectors(cf64.p, tail->uni, g.Nk, g.Norb);
    DBuf<cx<float>> cf32;
    const cx<T>* cf = nullptr;
    if constexpr (std::is_same<T, float>::value) {
      cf32.alloc(ncf);
      convert<float, double>(cf32.p, cf64.p, (long long)ncf);
      cf = cf32.p;
    } else {
      cf = cf64.p;
    }
    A.alloc((size_t)No2 * g.P);
    B.alloc((size_t)No2 * g.P);
    k_ref_tau<R, T><<<mesh_tau_grid(g.Nkall, g.M, No2), 256, 0, st>>>(A.p, B.p, gp.p, gm.p, cf, g.grid_irr.p, g.grid_flag.p, g.Nkall,
                                         g.Nk, g.Norb, (int)g.M, g.P);
    count_launch("ref_tau");
    fft.forward_space<R>(A.p, No2, st);
    fft.forward_space<R>(B.p, No2, st);
    DBuf<double2> rb(No2);
    k_rhobar<<<No2, 256, 0, st>>>(rb.p, tail->uni, ff.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Norb);
    count_launch("rhobar");
    std::vector<double2> hrb(No2);
    rb.download(hrb.data(), No2);
    sync();
    auto RB = [&](int m, int l) { return hrb[m + g.Norb * l]; };
    auto Jof = [&](int l, int m) {  // tau = 0 jump coefficient of pair (l,m) (fchi.f90:836-844)
      const int a13 = p.o1[l], b13 = p.o1[m], a42 = p.o2[m], b42 = p.o2[l];
      double2 J = make_double2(0, 0);
      if (a13 == b13) J = J + RB(a42, b42);
      if (a42 == b42) J = J - RB(a13, b13);
      return J;
    };
    for (auto& c : hp) {
      c.J = Jof(c.l, c.m);
      if (c.has_d) c.dJ = Jof(c.dl, c.dm);
    }
    // the sawtooth transform depends on (Nw, T) only: computed once per pair
    static std::map<std::pair<int, double>, DBuf<double2>*> sawc_cache;
    static std::mutex sawc_mu;
    const double2* sawc64 = nullptr;
    {
      std::lock_guard<std::mutex> lk(sawc_mu);
      DBuf<double2>*& e = sawc_cache[std::make_pair(g.Nw, temp)];
      if (!e) {
        e = new DBuf<double2>(g.Nw);
        k_sawc<<<grid_1d(g.Nw, 128), 128, 0, st>>>(e->p, g.Nw, (int)g.M, temp);
        count_launch("sawc");
        // complete before another thread's stream reads the cached entry
        PGB_CUDA(cudaStreamSynchronize(st));
      }
      sawc64 = e->p;
    }
    sawc.alloc(g.Nw);
    narrow<R>(sawc.p, sawc64, g.Nw);
  }
  {  // keep only the transforms that are computed
    std::vector<ChiDev> kept;
    for (size_t i = 0; i < hp.size(); ++i)
      if (derived[i] < 0) kept.push_back(hp[i]);
    hp.swap(kept);
  }
  DBuf<ChiDev> dp(hp.size());
  dp.upload(hp.data(), hp.size());
  PGB_CUDA(cudaMemsetAsync(chi, 0, sizeof(cx<R>) * (size_t)g.K * g.Nchi * g.Nchi, st));
  // chunk of pairs per backward batch: bounded by free memory
  sync();
  const size_t freeb = device_bytes_available();
  long long ch = (long long)((freeb / 3) / (sizeof(cx<R>) * (size_t)g.P));
  ch = std::max(1LL, std::min<long long>(ch, (long long)hp.size()));
  ch = std::min(ch, 64LL);
  DBuf<cx<R>> T((size_t)ch * g.P);
  const double sc = temp / (double)g.Nkall / (double)g.P;
  const double sr = 1.0 / (temp * (double)g.Nkall) / (double)g.P;
  for (long long c0 = 0; c0 < (long long)hp.size(); c0 += ch) {
    const int nc = (int)std::min<long long>(ch, (long long)hp.size() - c0);
    k_chi0_product<R><<<mesh_tau_grid(g.Nkall, g.M, nc), 256, 0, st>>>(T.p, F.p, tail ? F0.p : nullptr, tail ? A.p : nullptr,
                                          tail ? B.p : nullptr, dp.p + c0, g.P, g.Nx, g.Ny, g.Nz, (int)g.M,
                                          fft.d_rev(0), fft.d_rev(1), fft.d_rev(2), fft.d_rev(3),
                                          fft.d_logical(3), (R)sc, (R)sr);
    count_launch("chi0_product");
    fft.backward<R>(T.p, nc, st);
    k_chi0_scatter<R><<<mesh_tau_grid(g.Nk, g.Nw, nc), 256, 0, st>>>(chi, T.p, dp.p + c0, g.irr_grid.p, tail ? sawc.p : nullptr,
                                          g.Nkall, g.Nk, g.Nw, g.Nchi, g.P);
    count_launch("chi0_scatter");
  }
}

// ================================================================ stoner ==
// Largest real part of the eigenvalues of M = sg chi0(q,0) V (fchi.f90:352-399,
// zgeev there), one warp per matrix: the Householder reduction to Hessenberg
// form and the Wilkinson-shifted QR iteration of eigvals_general, with lane j
// owning column j in the left updates and row i in the right updates.  The
// matrix sits in shared memory with a padded row; every lane evaluates the
// scalar control flow (deflation, shifts, rotations) from shared memory, so
// it is warp-uniform.
constexpr int kStonerWarps = 4;
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float2 csqrt_f(float2 z) {
  const float r = hypotf(z.x, z.y);
  if (r == 0.0f) return mkc(0.0f, 0.0f);
  const float t = sqrtf(0.5f * (r + fabsf(z.x)));
  if (z.x >= 0) return mkc(t, z.y / (2 * t));
  return mkc(fabsf(z.y) / (2 * t), z.y >= 0 ? t : -t);
}
__device__ __forceinline__ double2 csqrt_t(double2 z) { return csqrt_(z); }
__device__ __forceinline__ float2 csqrt_t(float2 z) { return csqrt_f(z); }
template <typename T> constexpr T kEpsOf = (T)2.220446049250313e-16;
template <> constexpr float kEpsOf<float> = 1.1920929e-7f;
// T is the arithmetic of the reduction and the QR: double for every chi0
// type, float for an FP32 chi0 in the fast schedule (stoner() decides)
template <typename R, typename T>
__global__ void __launch_bounds__(32 * kStonerWarps) k_stoner(double* out, const cx<R>* chi, const double* S,
                                                              const double* C, int Nk, int Nw, int n, int* err) {
  using cT = cx<T>;
  extern __shared__ __align__(16) unsigned char sm_st[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ld = n + 1;
  cT* A = reinterpret_cast<cT*>(sm_st) + (size_t)w * (n * ld + 64);
  cT* v = A + n * ld;   // Householder vector / rotation sines
  T* cs = reinterpret_cast<T*>(v + 32);
  const int t = blockIdx.x * kStonerWarps + w;
  if (t >= 2 * Nk) return;  // warp-uniform
  const int k0 = t % Nk, which = t / Nk;
  const double* V = which ? C : S;
  const T sg = which ? (T)-1 : (T)1;
  const cT zero = cmk<T>((T)0, (T)0);
  if (lane < n) {
    for (int b = 0; b < n; ++b) {
      cT acc = zero;
      for (int c = 0; c < n; ++c) acc += (T)V[c + n * b] * ccast<T>(chi[fidx(k0, 0, lane, c, Nk, Nw, n)]);
      A[lane * ld + b] = sg * acc;
    }
  }
  __syncwarp();
  // Householder reduction to upper Hessenberg form
  for (int k = 0; k + 2 < n; ++k) {
    const T xn = sqrt(warp_sum<T>((lane > k && lane < n) ? abs2(A[lane * ld + k]) : (T)0));
    if (xn == 0) continue;
    const cT x0 = A[(k + 1) * ld + k];
    const T a0 = hypot(x0.x, x0.y);
    const cT ph = a0 > 0 ? cmk<T>(x0.x / a0, x0.y / a0) : cmk<T>((T)1, (T)0);
    const cT alpha = cmk<T>(-ph.x * xn, -ph.y * xn);
    cT vl = zero;
    if (lane > k && lane < n) vl = A[lane * ld + k] - ((lane == k + 1) ? alpha : zero);
    const T vn = warp_sum<T>(abs2(vl));
    if (lane < 32) v[lane] = vl;
    __syncwarp();
    if (vn == 0) continue;
    const T sc = (T)2 / vn;
    if (lane >= k && lane < n) {  // A = (I - sc v v^H) A, column j = lane
      cT s = zero;
      for (int i = k + 1; i < n; ++i) s += conj(v[i]) * A[i * ld + lane];
      s = sc * s;
      for (int i = k + 1; i < n; ++i) A[i * ld + lane] -= v[i] * s;
    }
    __syncwarp();
    if (lane < n) {  // A = A (I - sc v v^H), row i = lane
      cT s = zero;
      for (int j = k + 1; j < n; ++j) s += A[lane * ld + j] * v[j];
      s = sc * s;
      for (int j = k + 1; j < n; ++j) A[lane * ld + j] -= s * conj(v[j]);
      if (lane >= k + 2) A[lane * ld + k] = zero;
    }
    __syncwarp();
  }
  // shifted QR on the active block [l, hi]
  double best = -1e300;
  int hi = n - 1, iter = 0, total = 0;
  bool failed = false;
  const T eps = kEpsOf<T>;
  while (hi >= 0) {
    if (hi == 0) { best = fmax(best, (double)A[0].x); break; }
    int l = hi;
    while (l > 0) {
      T s = cabs1(A[(l - 1) * ld + l - 1]) + cabs1(A[l * ld + l]);
      if (s == 0) s = 1.0;
      if (cabs1(A[l * ld + l - 1]) <= eps * s) break;
      --l;
    }
    if (l == hi) {
      best = fmax(best, (double)A[hi * ld + hi].x);
      --hi;
      iter = 0;
      continue;
    }
    __syncwarp();
    if (l > 0 && lane == 0) A[l * ld + l - 1] = zero;
    __syncwarp();  // the exceptional shift may read the element just zeroed
    if (++iter > 60 || ++total > 60 * n) { failed = true; break; }
    cT mu;
    if (iter % 11 == 10) {  // exceptional shift
      const T e = cabs1(A[hi * ld + hi - 1]) + (hi >= 2 ? cabs1(A[(hi - 1) * ld + hi - 2]) : (T)0);
      mu = A[hi * ld + hi] + cmk<T>((T)0.75 * e, (T)0);
    } else {
      const cT a = A[(hi - 1) * ld + hi - 1], b = A[(hi - 1) * ld + hi];
      const cT c = A[hi * ld + hi - 1], d = A[hi * ld + hi];
      const cT hd = (T)0.5 * (a - d);
      const cT disc = csqrt_t(hd * hd + b * c);
      const cT m1 = (T)0.5 * (a + d) + disc, m2 = (T)0.5 * (a + d) - disc;
      mu = (abs2(m1 - d) < abs2(m2 - d)) ? m1 : m2;
    }
    __syncwarp();
    if (lane >= l && lane <= hi) A[lane * ld + lane] -= mu;
    __syncwarp();
    for (int k = l; k < hi; ++k) {
      const cT a = A[k * ld + k], b = A[(k + 1) * ld + k];
      const T aa = hypot(a.x, a.y), bb = hypot(b.x, b.y);
      const T r = hypot(aa, bb);
      T c;
      cT s;
      if (r == 0) { c = (T)1; s = zero; }
      else if (aa == 0) { c = (T)0; s = conj(b) * ((T)1 / bb); }
      else { c = aa / r; s = cmk<T>(a.x / aa, a.y / aa) * conj(b) * ((T)1 / r); }
      if (lane == 0) { cs[k] = c; v[k] = s; }
      __syncwarp();
      if (lane >= k && lane <= hi) {
        const cT x = A[k * ld + lane], y = A[(k + 1) * ld + lane];
        A[k * ld + lane] = c * x + s * y;
        A[(k + 1) * ld + lane] = c * y - conj(s) * x;
      }
      __syncwarp();
    }
    for (int k = l; k < hi; ++k) {
      const T c = cs[k];
      const cT s = v[k];
      const int imax = (k + 2 < hi) ? k + 2 : hi;
      if (lane >= l && lane <= imax) {
        const cT x = A[lane * ld + k], y = A[lane * ld + k + 1];
        A[lane * ld + k] = c * x + y * conj(s);
        A[lane * ld + k + 1] = c * y - x * s;
      }
      __syncwarp();
    }
    if (lane >= l && lane <= hi) A[lane * ld + lane] += mu;
    __syncwarp();
  }
  if (lane == 0) {
    if (failed) atomicExch(err, 2);
    out[t] = best;
  }
}

// false if the QR of some matrix did not converge
template <typename R, typename T>
bool stoner_launch(const Geom& g, const cx<R>* chi, const double* S, const double* C, std::vector<double>& h) {
  reset_err();
  DBuf<double> out(2 * (size_t)g.Nk);
  const size_t smem = (size_t)kStonerWarps * ((size_t)g.Nchi * (g.Nchi + 1) + 64) * sizeof(cx<T>);
  PGB_SMEM_LIMIT_ONCE((k_stoner<R, T>), 96 * 1024);
  const unsigned blocks = (unsigned)((2LL * g.Nk + kStonerWarps - 1) / kStonerWarps);
  k_stoner<R, T><<<blocks, 32 * kStonerWarps, smem, ctx().stream>>>(out.p, chi, S, C, g.Nk, g.Nw, g.Nchi,
                                                                     ctx().err);
  count_launch("stoner");
  h.resize(2 * (size_t)g.Nk);
  out.download(h.data(), h.size());
  return fetch_err() == 0;
}

// max Re eig of chi0(q,0) S and -chi0(q,0) C over q (fchi.f90:352-399).  An
// FP32 chi0 carries about 1e-7 relative rounding, so its QR runs in FP32 on
// the FP32 pipe (64 times the FP64 rate); it is redone in FP64 when the FP32
// Stoner factor lies within 1e-3 of 1, where the sw_rescale clamp decides.
template <typename R>
void stoner(const Geom& g, const cx<R>* chi, const double* S, const double* C, double* sdw, double* cdw,
            int* q_sdw, int* q_cdw) {
  std::vector<double> h;
  bool done = false;
  if constexpr (std::is_same<R, float>::value) {
    if (stoner_launch<R, float>(g, chi, S, C, h)) {
      double s32 = -1.0e5;
      for (int k = 0; k < g.Nk; ++k) s32 = std::max(s32, h[k]);
      done = std::fabs(s32 - 1.0) >= 1.0e-3;
    }
  }
  if (!done)
    PGB_CHECK((stoner_launch<R, double>(g, chi, S, C, h)), "eigenvalue iteration of chi0(q,0)S did not converge");
  double s2 = -1.0e5, c2 = -1.0e5;
  int qs = 0, qc = 0;
  for (int k = 0; k < g.Nk; ++k) {
    if (h[k] > s2) { s2 = h[k]; qs = k; }
    if (h[g.Nk + k] > c2) { c2 = h[g.Nk + k]; qc = k; }
  }
  *sdw = s2;
  *cdw = c2;
  if (q_sdw) *q_sdw = qs;
  if (q_cdw) *q_cdw = qc;
}

void ckchi_print(const Geom& g, double sdw, double cdw, int qs, int qc) {
  auto kc = [&](int k, int c) { return (long long)g.h_kmap[3 * (long long)g.h_full_of_grid[g.h_irr_grid[k]] + c]; };
  log("SDW%4lld%4lld%4lld%12.8f\n", kc(qs, 0), kc(qs, 1), kc(qs, 2), sdw);
  log("CDW%4lld%4lld%4lld%12.8f\n", kc(qc, 0), kc(qc, 1), kc(qc, 2), cdw);
}
void ckchi_print_soc(const Geom& g, double v, int q) {  // fchi0withsoc.f90:189-197
  auto kc = [&](int c) { return (long long)g.h_kmap[3 * (long long)g.h_full_of_grid[g.h_irr_grid[q]] + c]; };
  log("SDW/CDW%4lld%4lld%4lld%12.8f\n", kc(0), kc(1), kc(2), v);
}

// ================================================================ vertex ==
template <typename R>
__global__ void k_vertex(cx<R>* chi, long long nmat, long long mstride, long long estride, int n,
                         const double* S, const double* C, int mode, int warps, int* err) {
  extern __shared__ __align__(16) unsigned char sm[];
  double* sS = reinterpret_cast<double*>(sm);
  double* sC = sS + n * n;
  double* sSC = sC + n * n;
  size_t off = ((size_t)3 * n * n * sizeof(double) + 15) / 16 * 16;
  cx<R>* wb = reinterpret_cast<cx<R>*>(sm + off);
  const int ld = n;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  cx<R>* X = wb + (size_t)w * 4 * n * ld;
  cx<R>* Pm = X + n * ld;
  cx<R>* Q = Pm + n * ld;
  cx<R>* T = Q + n * ld;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int a = e / n, b = e % n;
    sS[a * n + b] = S[a + n * b];
    sC[a * n + b] = C[a + n * b];
    sSC[a * n + b] = S[a + n * b] + C[a + n * b];
  }
  __syncthreads();
  for (long long mat = (long long)blockIdx.x * warps + w; mat < nmat; mat += (long long)gridDim.x * warps) {
    cx<R>* base = chi + mat * mstride;
    for (int e = lane; e < n * n; e += 32) X[(e % n) * ld + e / n] = base[estride * e];
    __syncwarp();
    wmm_cr<R>(Pm, X, sS, n, ld, (R)1);  // chi0 S
    wmm_cr<R>(Q, X, sC, n, ld, (R)1);   // chi0 C
    bool ok = true;
    if (mode == 0) {
      // V = 1.5S - 0.5C - 0.25 (S+C)(chi0S + chi0C) + 1.5 S Xs + 0.5 C Xc
      if (lane < n)
        for (int j = 0; j < n; ++j) {
          cx<R> acc = cmk<R>(0, 0);
          for (int k = 0; k < n; ++k) acc += (R)sSC[lane * n + k] * (Pm[k * ld + j] + Q[k * ld + j]);
          X[lane * ld + j] = cmk<R>((R)(1.5 * sS[lane * n + j] - 0.5 * sC[lane * n + j]), (R)0) - (R)0.25 * acc;
        }
      __syncwarp();
    } else if (mode == 1 || mode == 2) {
      const double sg = (mode == 1) ? 1.0 : -1.0;
      for (int e = lane; e < n * n; e += 32)
        X[(e / n) * ld + e % n] = cmk<R>((R)(0.5 * (sS[e] + sg * sC[e])), (R)0);
      __syncwarp();
    }
    if (mode <= 2) {
      // T = I - chi0 S ; solve T Xs = chi0 S
      for (int e = lane; e < n * n; e += 32) {
        const int a = e / n, b = e % n;
        T[a * ld + b] = cmk<R>((R)(a == b), (R)0) - Pm[a * ld + b];
      }
      __syncwarp();
      ok &= wsolve<R>(T, Pm, n, ld);
      const R cs = (mode == 2) ? (R)-0.5 : (R)1.5;
      wmm_rc_acc<R>(X, sS, Pm, n, ld, cs);
      for (int e = lane; e < n * n; e += 32) {
        const int a = e / n, b = e % n;
        T[a * ld + b] = cmk<R>((R)(a == b), (R)0) + Q[a * ld + b];
      }
      __syncwarp();
      ok &= wsolve<R>(T, Q, n, ld);
      const R cc = (mode == 0) ? (R)0.5 : (R)-0.5;
      wmm_rc_acc<R>(X, sC, Q, n, ld, cc);
    } else {
      // chi_s = (I - chi0 S)^-1 chi0 (mode 3), chi_c = (I + chi0 C)^-1 chi0 (mode 4)
      for (int e = lane; e < n * n; e += 32) {
        const int a = e / n, b = e % n;
        T[a * ld + b] = cmk<R>((R)(a == b), (R)0) + ((mode == 3) ? -Pm[a * ld + b] : Q[a * ld + b]);
      }
      __syncwarp();
      ok &= wsolve<R>(T, X, n, ld);
    }
    if (!ok && lane == 0) atomicExch(err, 3);
    for (int e = lane; e < n * n; e += 32) base[estride * e] = X[(e % n) * ld + e / n];
    __syncwarp();
  }
}

// Register-resident vertex for Nchi in {1,4,9,16,25}: lane i holds row i.
// With Si = S^-1, Ci = C^-1 (computed once on the host):
//   S (I - chi0 S)^-1 = (Si - chi0)^-1,   C (I + chi0 C)^-1 = (Ci + chi0)^-1,
// so (fUJ.f90:253-365)
//   V_sigma         = 1.5 (Si - X)^-1 - 0.5 (Ci + X)^-1 - 0.25 (S+C) X (S+C)
//   V_Delta singlet = -S + 1.5 (Si - X)^-1 + 0.5 (Ci + X)^-1
//   V_Delta triplet = S - C - 0.5 (Si - X)^-1 + 0.5 (Ci + X)^-1
// Each inverse is an in-place Gauss-Jordan elimination with partial pivoting
// (|Re|+|Im|, first maximum); row interchanges relabel lanes instead of
// moving data, and the pivot row is broadcast with warp shuffles.
template <typename R, int N>
__device__ __forceinline__ cx<R> pick(const cx<R> (&a)[N], int k) {
  cx<R> v = a[0];
#pragma unroll
  for (int j = 1; j < N; ++j)
    if (j == k) v = a[j];
  return v;
}

// The elimination step loop is kept rolled (register entries selected by
// comparison, not by dynamic indexing): a fully unrolled 25x25 elimination
// is tens of thousands of straight-line instructions per matrix and runs
// from the instruction cache's backing store.
template <typename R, int N>
__device__ __forceinline__ bool warp_inverse(cx<R> (&a)[N], int* piv, int* map) {
  const int lane = threadIdx.x & 31;
  int label = lane;
  bool ok = true;
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    const cx<R> ak = pick<R, N>(a, k);
    R v = (lane < N && label >= k) ? cabs1(ak) : (R)-1;
    int key = (lane < N && label >= k) ? label : 1 << 20;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const R ov = shfl_xor(v, off);
      const int ok2 = __shfl_xor_sync(0xffffffffu, key, off);
      if (ov > v || (ov == v && ok2 < key)) { v = ov; key = ok2; }
    }
    const int plabel = key;
    if (!(v > 0)) ok = false;
    if (label == k) label = plabel;
    else if (label == plabel) label = k;
    if (lane == 0) piv[k] = plabel;
    const unsigned m = __ballot_sync(0xffffffffu, label == k && lane < N);
    const int src = __ffs(m) - 1;
    const cx<R> pv = cmk<R>(shfl_idx(ak.x, src), shfl_idx(ak.y, src));
    const cx<R> ip = ok ? cdiv(cmk<R>(1, 0), pv) : cmk<R>(0, 0);
    const bool is_piv = (label == k);
    // new row = base + f * (pivot row): the pivot lane scales (base 0, f = 1/p),
    // the others eliminate (base = own row, f = -a_k/p); column k becomes f
    const cx<R> f = is_piv ? ip : -(ak * ip);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const R sx = shfl_idx(a[j].x, src), sy = shfl_idx(a[j].y, src);
      const R bx = is_piv ? (R)0 : a[j].x, by = is_piv ? (R)0 : a[j].y;
      const cx<R> nv = cmk<R>(mad(f.x, sx, mad(-f.y, sy, bx)), mad(f.x, sy, mad(f.y, sx, by)));
      a[j] = (j == k) ? f : nv;
    }
  }
  __syncwarp();
  // undo the interchanges: columns in reverse order
#pragma unroll 1
  for (int k = N - 1; k >= 0; --k) {
    const int p = piv[k];
    if (p != k) {
      const cx<R> ak = pick<R, N>(a, k), ap = pick<R, N>(a, p);
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = (j == k) ? ap : ((j == p) ? ak : a[j]);
    }
  }
  // bring logical row i back to lane i
  if (lane < N) map[label] = lane;
  __syncwarp();
  const int from = (lane < N) ? map[lane] : lane;
#pragma unroll
  for (int j = 0; j < N; ++j) a[j] = cmk<R>(shfl_idx(a[j].x, from), shfl_idx(a[j].y, from));
  __syncwarp();
  return ok;
}

// Pivot magnitude |Re| + |Im| as a float, for the pivot key of
// warp_inverse_rot (double-float: the high words)
__device__ __forceinline__ float pivot_mag(float2 a) { return fabsf(a.x) + fabsf(a.y); }
__device__ __forceinline__ float pivot_mag(double2 a) { return (float)(fabs(a.x) + fabs(a.y)); }
__device__ __forceinline__ float pivot_mag(cdf a) { return fabsf(a.x.hi) + fabsf(a.y.hi); }

// Shared pivot row of warp_inverse_rot.  FP32 entries are stored one place
// up (slot s at index s + 1), so that slots 1..N-1 pair into aligned 16-byte
// words: one store per two entries for the pivot lane, one broadcast load
// per two entries for the others.  16-byte entries are stored at index s.
template <typename C> __host__ __device__ constexpr int prow_len(int n) { return sizeof(C) == 8 ? ((n + 2) & ~1) : n; }

template <int N> __device__ __forceinline__ void prow_put(float2* d, const float2 (&a)[N]) {
  float4* d4 = reinterpret_cast<float4*>(d);
  d[1] = a[0];
#pragma unroll
  for (int s = 1; s < N; s += 2) {
    if (s + 1 < N) d4[(s + 1) >> 1] = make_float4(a[s].x, a[s].y, a[s + 1].x, a[s + 1].y);
    else d[s + 1] = a[s];
  }
}
template <typename C, int N> __device__ __forceinline__ void prow_put(C* d, const C (&a)[N]) {
#pragma unroll
  for (int s = 0; s < N; ++s) d[s] = a[s];
}
__device__ __forceinline__ float2 prow_pivot(const float2* d) { return d[1]; }
template <typename C> __device__ __forceinline__ C prow_pivot(const C* d) { return d[0]; }

// Gauss-Jordan inverse of the warp's matrix (lane = row, N complex entries
// in registers), arranged so that a step is little more than its complex
// FMAs:
//  * the column being eliminated always sits in register slot 0: a step
//    writes its update of slot s into slot s - 1 and the new column into
//    slot N - 1, so no register is ever indexed by the step number, and after
//    N steps the slots are back in order;
//  * the pivot row of a step is not divided by its pivot: it stays as it is
//    and its entry of the eliminated column becomes 1.  Row r of the inverse
//    is then the register row times 1 / (its pivot), which is returned in
//    `scale` for the caller to fold into its write.  The other rows are
//    eliminated with f = -a_k / p as in the textbook form, so every row
//    equals the textbook row times a constant, and the pivot choices are
//    the same;
//  * the pivot row reaches the other lanes through shared memory (a
//    double buffer `prow` of 2 x prow_len entries per warp) instead of two
//    shuffles per entry;
//  * the pivot is the candidate row with the largest |Re| + |Im|, taken by one
//    redux.sync over a key of the magnitude's top 27 bits and the row label
//    (the lowest label among equal keys; magnitudes within 2^-18 of each
//    other count as equal).
// Row interchanges relabel lanes (the lane holds logical row `label`), and
// column interchanges are not undone in registers: on return pos[c] (per
// warp, shared) is the column of the inverse that register slot c holds, for
// rows with lane < N.  piv[] (N ints, shared) is scratch.
template <typename R, int N>
__device__ __forceinline__ bool warp_inverse_rot(cx<R> (&a)[N], cx<R>* prow, int* piv, int* pos, int& label,
                                                 cx<R>& scale) {
  constexpr int PL = prow_len<cx<R>>(N);
  const int lane = threadIdx.x & 31;
  label = lane;
  scale = cmk<R>((R)0, (R)0);
  bool ok = true;
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    const cx<R> ak = a[0];
    unsigned key = 0u;
    if (lane < N && label >= k) key = (__float_as_uint(pivot_mag(ak)) & ~31u) | (unsigned)(31 - label);
    const unsigned best = __reduce_max_sync(0xffffffffu, key);
    const int plabel = 31 - (int)(best & 31u);
    if (!(__uint_as_float(best & ~31u) > 0.f)) ok = false;
    const bool is_piv = (label == plabel);
    if (label == k) label = plabel;
    else if (is_piv) label = k;
    if (lane == 0) piv[k] = plabel;
    cx<R>* buf = prow + (k & 1) * PL;
    if (is_piv) prow_put(buf, a);
    __syncwarp();
    const cx<R> p = prow_pivot(buf);
    const cx<R> ip = ok ? crecip(p) : cmk<R>((R)0, (R)0);
    if (is_piv) scale = ip;
    const cx<R> f = is_piv ? cmk<R>((R)0, (R)0) : -(ak * ip);
    if constexpr (sizeof(cx<R>) == 8) {
      const float4* b4 = reinterpret_cast<const float4*>(buf);
#pragma unroll
      for (int s = 1; s < N; s += 2) {
        const float4 q = b4[(s + 1) >> 1];
        a[s - 1] = cmk<R>(mad(f.x, q.x, mad(-f.y, q.y, a[s].x)), mad(f.x, q.y, mad(f.y, q.x, a[s].y)));
        if (s + 1 < N)
          a[s] = cmk<R>(mad(f.x, q.z, mad(-f.y, q.w, a[s + 1].x)), mad(f.x, q.w, mad(f.y, q.z, a[s + 1].y)));
      }
    } else {
#pragma unroll
      for (int s = 1; s < N; ++s) {
        const cx<R> q = buf[s];
        a[s - 1] = cmk<R>(mad(f.x, q.x, mad(-f.y, q.y, a[s].x)), mad(f.x, q.y, mad(f.y, q.x, a[s].y)));
      }
    }
    a[N - 1] = is_piv ? cmk<R>((R)1, (R)0) : f;
  }
  // the column interchanges, in reverse order, applied to the position of
  // register slot `lane`
  __syncwarp();
  if (lane < N) {
    int c = lane;
#pragma unroll 1
    for (int k = N - 1; k >= 0; --k) {
      const int p = piv[k];
      if (c == k) c = p;
      else if (c == p) c = k;
    }
    pos[lane] = c;
  }
  __syncwarp();
  return ok;
}

// Matrices of consecutive (q,iv) are staged through shared memory in tiles of
// 2W: the loads and stores of the Fortran (Nk,Nw,Nchi,Nchi) layout are then
// runs of 2W consecutive elements instead of one element per cache sector.
template <typename R, int N, int W>
__global__ void __launch_bounds__(32 * W) k_vertex_reg(cx<R>* chi, long long nmat, long long estride,
                                                       const R* consts, int mode, int* err) {
  constexpr int T = 2 * W;          // matrices per tile
  constexpr int TP = T + 1;         // padded tile row
  extern __shared__ __align__(16) unsigned char smraw[];
  // constants in the compute precision: an FP64->FP32 conversion per use
  // would run on the FP64 pipe
  R* cs = reinterpret_cast<R*>(smraw);                                 // Si, Ci, S+C, S, C
  constexpr size_t cs_bytes = (5 * N * N * sizeof(R) + 15) / 16 * 16;  // keep the tile 16-byte aligned
  cx<R>* tile = reinterpret_cast<cx<R>*>(smraw + cs_bytes);            // [N*N][TP]
  cx<R>* tb = tile + (size_t)N * N * TP;                               // [W][N*N]
  int* pv = reinterpret_cast<int*>(tb + (size_t)W * N * N);            // [W][N+1]
  int* mp = pv + W * (N + 1);                                          // [W][32]
  for (int e = threadIdx.x; e < 5 * N * N; e += blockDim.x) cs[e] = consts[e];
  const R* Si = cs;
  const R* Ci = cs + N * N;
  const R* SC = cs + 2 * N * N;
  const R* Sm = cs + 3 * N * N;
  const R* Cm = cs + 4 * N * N;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = lane < N ? lane : 0;
  cx<R>* tbw = tb + (size_t)w * N * N;
  const R c1 = mode == 2 ? (R)-0.5 : (R)1.5;
  const R c2 = mode == 0 ? (R)-0.5 : (R)0.5;
  for (long long m0 = (long long)blockIdx.x * T; m0 < nmat; m0 += (long long)gridDim.x * T) {
    const int nt = (int)min((long long)T, nmat - m0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < N * N * T; idx += blockDim.x) {
      const int t = idx % T, e = idx / T;
      if (t < nt) tile[e * TP + t] = chi[m0 + t + estride * e];
    }
    __syncthreads();
    for (int t = w; t < nt; t += W) {
      // x(i, j) = tile[(i + N j) * TP + t]
      cx<R> a[N], v[N];
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = cmk<R>((R)Si[i * N + j], (R)0) - tile[(i + N * j) * TP + t];
      bool ok = warp_inverse<R, N>(a, pv + w * (N + 1), mp + w * 32);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        R base = 0;
        if (mode == 1) base = (R)-Sm[i * N + j];
        else if (mode == 2) base = (R)(Sm[i * N + j] - Cm[i * N + j]);
        v[j] = cmk<R>(base, (R)0) + c1 * a[j];
      }
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = cmk<R>((R)Ci[i * N + j], (R)0) + tile[(i + N * j) * TP + t];
      ok &= warp_inverse<R, N>(a, pv + w * (N + 1), mp + w * 32);
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] += c2 * a[j];
      if (mode == 0) {
        // -0.25 (S+C) X (S+C): t = X (S+C) row-local, then (S+C) t through smem
#pragma unroll
        for (int j = 0; j < N; ++j) a[j] = cmk<R>(0, 0);
#pragma unroll 1
        for (int k = 0; k < N; ++k) {
          const cx<R> xk = tile[(i + N * k) * TP + t];
#pragma unroll
          for (int j = 0; j < N; ++j) a[j] += SC[k * N + j] * xk;
        }
        if (lane < N) {
#pragma unroll
          for (int j = 0; j < N; ++j) tbw[i * N + j] = a[j];
        }
        __syncwarp();
#pragma unroll 1
        for (int k = 0; k < N; ++k) {
          const R sk = (R)-0.25 * SC[i * N + k];
#pragma unroll
          for (int j = 0; j < N; ++j) v[j] += sk * tbw[k * N + j];
        }
      }
      if (!ok && lane == 0) atomicExch(err, 3);
      __syncwarp();
      if (lane < N) {
#pragma unroll
        for (int j = 0; j < N; ++j) tile[(i + N * j) * TP + t] = v[j];
      }
      __syncwarp();
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < N * N * T; idx += blockDim.x) {
      const int t = idx % T, e = idx / T;
      if (t < nt) chi[m0 + t + estride * e] = tile[e * TP + t];
    }
  }
}

// Register vertex with the output accumulated in shared memory: one row of
// the working matrix (N complex values) is the only per-lane register array,
// so N = 25 fits in FP64.  One matrix per warp per tile.  The tile slot of a
// matrix holds X until both inversions are done, then X(S+C) as the scratch
// of the sandwich term, then the result.  The inversions are
// warp_inverse_rot's: each lane writes its register row, times the row's
// scale, to the accumulator at the row's label and the slots' columns.
template <typename R, int N, int W>
__global__ void __launch_bounds__(32 * W, (sizeof(R) == 4 ? 2 : 1)) k_vertex_vs(cx<R>* chi, long long nmat,
                                                                                 long long estride,
                                                      const R* consts, int mode, int* err) {
  constexpr int T = W;
  constexpr int TP = T + 1;
  constexpr int PL = prow_len<cx<R>>(N);
  extern __shared__ __align__(16) unsigned char smraw[];
  // Si, Ci and S+C in shared memory; S and C (the V_Delta modes' constant
  // parts) from global memory through the read-only cache
  R* cs = reinterpret_cast<R*>(smraw);
  constexpr size_t cs_bytes = (3 * N * N * sizeof(R) + 15) / 16 * 16;
  cx<R>* prow = reinterpret_cast<cx<R>*>(smraw + cs_bytes);  // [W][2][PL] pivot rows
  cx<R>* tile = prow + (size_t)W * 2 * PL;                    // [N*N][TP]
  cx<R>* vb = tile + (size_t)N * N * TP;                      // [W][N][N], entry (r, c) at c * N + r
  int* pv = reinterpret_cast<int*>(vb + (size_t)W * N * N);   // [W][N+1]
  int* ps = pv + W * (N + 1);                                 // [W][32]
  for (int e = threadIdx.x; e < 3 * N * N; e += blockDim.x) cs[e] = consts[e];
  const R* Si = cs;
  const R* Ci = cs + N * N;
  const R* SC = cs + 2 * N * N;
  const R* Sm = consts + 3 * N * N;
  const R* Cm = consts + 4 * N * N;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = lane < N ? lane : 0;
  const bool row = lane < N;
  cx<R>* vw = vb + (size_t)w * N * N;
  cx<R>* pw = prow + (size_t)w * 2 * PL;
  int* pvw = pv + w * (N + 1);
  int* psw = ps + w * 32;
  const R c1 = mode == 2 ? (R)-0.5 : (R)1.5;
  const R c2 = mode == 0 ? (R)-0.5 : (R)0.5;
  for (long long m0 = (long long)blockIdx.x * T; m0 < nmat; m0 += (long long)gridDim.x * T) {
    const int nt = (int)min((long long)T, nmat - m0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < N * N * T; idx += blockDim.x) {
      const int t = idx % T, e = idx / T;
      if (t < nt) tile[e * TP + t] = chi[m0 + t + estride * e];
    }
    __syncthreads();
    const int t = w;
    if (t < nt) {
      cx<R> a[N];
      int lab;
      cx<R> sc;
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = cmk<R>(Si[i * N + j], (R)0) - tile[(i + N * j) * TP + t];
      bool ok = warp_inverse_rot<R, N>(a, pw, pvw, psw, lab, sc);
      if (row) {
        const cx<R> s1 = c1 * sc;
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const int c = psw[j];
          R base = 0;
          if (mode == 1) base = -Sm[lab * N + c];
          else if (mode == 2) base = Sm[lab * N + c] - Cm[lab * N + c];
          vw[c * N + lab] = cmk<R>(base, (R)0) + s1 * a[j];
        }
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = cmk<R>(Ci[i * N + j], (R)0) + tile[(i + N * j) * TP + t];
      ok &= warp_inverse_rot<R, N>(a, pw, pvw, psw, lab, sc);
      if (row) {
        const cx<R> s2 = c2 * sc;
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const int c = psw[j];
          vw[c * N + lab] += s2 * a[j];
        }
      }
      if (mode == 0) {
        // -0.25 (S+C) X (S+C): row i of X (S+C) into the tile slot, then (S+C) times it
#pragma unroll
        for (int j = 0; j < N; ++j) a[j] = cmk<R>(0, 0);
#pragma unroll 1
        for (int k = 0; k < N; ++k) {
          const cx<R> xk = tile[(i + N * k) * TP + t];
#pragma unroll
          for (int j = 0; j < N; ++j) a[j] += SC[k * N + j] * xk;
        }
        __syncwarp();
        if (lane < N) {
#pragma unroll
          for (int j = 0; j < N; ++j) tile[(i + N * j) * TP + t] = a[j];
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < N; ++j) a[j] = cmk<R>(0, 0);
#pragma unroll 1
        for (int k = 0; k < N; ++k) {
          const R sk = (R)-0.25 * SC[i * N + k];
#pragma unroll
          for (int j = 0; j < N; ++j) a[j] += sk * tile[(k + N * j) * TP + t];
        }
        if (row) {
#pragma unroll
          for (int j = 0; j < N; ++j) vw[j * N + lane] += a[j];
        }
      }
      if (!ok && lane == 0) atomicExch(err, 3);
      __syncwarp();
      if (lane < N) {
#pragma unroll
        for (int j = 0; j < N; ++j) tile[(i + N * j) * TP + t] = vw[j * N + lane];
      }
      __syncwarp();
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < N * N * T; idx += blockDim.x) {
      const int t2 = idx % T, e = idx / T;
      if (t2 < nt) chi[m0 + t2 + estride * e] = tile[e * TP + t2];
    }
  }
}

template <typename R, int N, int W> size_t vertex_vs_smem() {
  return (sizeof(R) * 3 * N * N + 15) / 16 * 16 + sizeof(cx<R>) * (size_t)W * 2 * prow_len<cx<R>>(N) +
         sizeof(cx<R>) * ((size_t)N * N * (W + 1) + (size_t)W * N * N) + sizeof(int) * (W * (N + 1) + W * 32);
}

template <typename R, int N, int W> size_t vertex_reg_smem() {
  return (sizeof(R) * 5 * N * N + 15) / 16 * 16 + sizeof(cx<R>) * ((size_t)N * N * (2 * W + 1) + (size_t)W * N * N) +
         sizeof(int) * (W * (N + 1) + W * 32);
}

// host inverse of a small real matrix (row-major), false if (nearly) singular
bool host_inverse(std::vector<double>& A, int n) {
  std::vector<int> piv(n);
  double amax = 0;
  for (double v : A) amax = std::max(amax, std::fabs(v));
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(A[r * n + k]) > std::fabs(A[p * n + k])) p = r;
    piv[k] = p;
    if (std::fabs(A[p * n + k]) <= 1e-12 * std::max(amax, 1e-300)) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
    const double d = 1.0 / A[k * n + k];
    A[k * n + k] = 1.0;
    for (int j = 0; j < n; ++j) A[k * n + j] *= d;
    for (int r = 0; r < n; ++r) {
      if (r == k) continue;
      const double f = A[r * n + k];
      A[r * n + k] = 0.0;
      for (int j = 0; j < n; ++j) A[r * n + j] -= f * A[k * n + j];
    }
  }
  for (int k = n - 1; k >= 0; --k)
    if (piv[k] != k)
      for (int r = 0; r < n; ++r) std::swap(A[r * n + k], A[r * n + piv[k]]);
  return true;
}

template <typename R, int N>
bool vertex_reg_launch(cx<R>* chi, long long nmat, long long estride, const R* dconsts, int mode) {
  constexpr int warps = (N >= 16) ? 4 : 8;
  const size_t smem = vertex_reg_smem<R, N, warps>();
  PGB_SMEM_LIMIT_ONCE((k_vertex_reg<R, N, warps>), smem);
  const long long tiles = (nmat + 2 * warps - 1) / (2 * warps);
  const long long blocks = std::min<long long>(tiles, (long long)ctx().num_sms * 8);
  k_vertex_reg<R, N, warps><<<(unsigned)std::max(1LL, blocks), 32 * warps, smem, ctx().stream>>>(
      chi, nmat, estride, dconsts, mode, ctx().err);
  count_launch("vertex_reg");
  return true;
}

template <typename R, int N>
bool vertex_vs_launch(cx<R>* chi, long long nmat, long long estride, const R* dconsts, int mode) {
  // FP32: 8 warps a CTA held to 128 registers (no spills), two CTAs and 16
  // warps per SM against 12 with 168 registers.  8-byte types: 4 warps at up
  // to 255 registers, so that two CTAs (8 warps) fit an SM in registers and
  // in shared memory (about 105 KB each for N = 25)
  constexpr int warps = sizeof(R) == 4 ? 8 : 4;
  const size_t smem = vertex_vs_smem<R, N, warps>();
  PGB_SMEM_LIMIT_ONCE((k_vertex_vs<R, N, warps>), smem);
  const long long tiles = (nmat + warps - 1) / warps;
  const long long blocks = std::min<long long>(tiles, (long long)ctx().num_sms * 8);
  k_vertex_vs<R, N, warps><<<(unsigned)std::max(1LL, blocks), 32 * warps, smem, ctx().stream>>>(chi, nmat, estride,
                                                                                                dconsts, mode, ctx().err);
  count_launch("vertex_vs");
  return true;
}

// FP32, N = 25: the shared-memory-accumulator kernel (default; 3.66 ms
// against 4.21 ms for 66,560 matrices, from 12 instead of 8 resident warps)
// or, with PYRPA_GB_VERTEX=reg, the all-register one
bool vertex_fp32_vs() {
  const char* s = std::getenv("PYRPA_GB_VERTEX");
  return !(s && std::string(s) == "reg");
}

template <typename R>
bool vertex(cx<R>* chi, long long nmat, long long stride, int Nchi, const double* S, const double* C,
            int mode) {
  // stride: distance between the elements of one matrix (matrices are consecutive, mstride 1)
  // stride < 0 selects compact matrices: mstride = Nchi^2, estride = 1
  long long mstride = 1, estride = stride;
  if (stride < 0) { mstride = (long long)Nchi * Nchi; estride = 1; }
  const int n = Nchi;
  const bool reg_size = (n == 1 || n == 4 || n == 9 || n == 16 || n == 25);
  if (mode <= 2 && reg_size && mstride == 1) {
    std::vector<double> hS(n * n), hC(n * n);
    PGB_CUDA(cudaMemcpyAsync(hS.data(), S, sizeof(double) * n * n, cudaMemcpyDeviceToHost, ctx().stream));
    PGB_CUDA(cudaMemcpyAsync(hC.data(), C, sizeof(double) * n * n, cudaMemcpyDeviceToHost, ctx().stream));
    sync();
    // row-major copies: element (a,b) of a Fortran (n,n) matrix is at a + n*b
    std::vector<double> Sr(n * n), Cr(n * n);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) {
        Sr[a * n + b] = hS[a + n * b];
        Cr[a * n + b] = hC[a + n * b];
      }
    std::vector<double> Si(Sr), Ci(Cr);
    if (host_inverse(Si, n) && host_inverse(Ci, n)) {
      std::vector<R> consts(5 * n * n);
      for (int e = 0; e < n * n; ++e) {
        consts[e] = (R)Si[e];
        consts[n * n + e] = (R)Ci[e];
        consts[2 * n * n + e] = (R)(Sr[e] + Cr[e]);
        consts[3 * n * n + e] = (R)Sr[e];
        consts[4 * n * n + e] = (R)Cr[e];
      }
      DBuf<R> dc(consts.size());
      dc.upload(consts.data(), consts.size());
      reset_err();
      if constexpr (std::is_same<R, dfl>::value) {
        switch (n) {
          case 1: vertex_vs_launch<R, 1>(chi, nmat, estride, dc.p, mode); break;
          case 4: vertex_vs_launch<R, 4>(chi, nmat, estride, dc.p, mode); break;
          case 9: vertex_vs_launch<R, 9>(chi, nmat, estride, dc.p, mode); break;
          case 16: vertex_vs_launch<R, 16>(chi, nmat, estride, dc.p, mode); break;
          case 25: vertex_vs_launch<R, 25>(chi, nmat, estride, dc.p, mode); break;
        }
        return fetch_err() == 0;
      }
      switch (n) {
        case 1: vertex_reg_launch<R, 1>(chi, nmat, estride, dc.p, mode); break;
        case 4: vertex_reg_launch<R, 4>(chi, nmat, estride, dc.p, mode); break;
        case 9: vertex_reg_launch<R, 9>(chi, nmat, estride, dc.p, mode); break;
        case 16:
          if constexpr (sizeof(R) == 4) vertex_reg_launch<R, 16>(chi, nmat, estride, dc.p, mode);
          else vertex_vs_launch<R, 16>(chi, nmat, estride, dc.p, mode);
          break;
        case 25:
          if constexpr (sizeof(R) == 4) {
            if (vertex_fp32_vs()) vertex_vs_launch<R, 25>(chi, nmat, estride, dc.p, mode);
            else vertex_reg_launch<R, 25>(chi, nmat, estride, dc.p, mode);
          } else {
            vertex_vs_launch<R, 25>(chi, nmat, estride, dc.p, mode);
          }
          break;
      }
      return fetch_err() == 0;
    }
  }
  if constexpr (std::is_same<R, dfl>::value) {
    throw Error("the double-float vertex supports Nchi = 1, 4, 9, 16 or 25 with invertible S and C");
  } else {
  const size_t head = ((size_t)3 * n * n * sizeof(double) + 15) / 16 * 16;
  const size_t per_warp = (size_t)4 * n * n * sizeof(cx<R>);
  int warps = (int)std::max<size_t>(1, std::min<size_t>(8, (200 * 1024 - head) / per_warp));
  const size_t smem = head + warps * per_warp;
  PGB_SMEM_LIMIT_ONCE(k_vertex<R>, 210 * 1024);
  reset_err();
  const long long blocks = std::min<long long>((nmat + warps - 1) / warps, (long long)ctx().num_sms * 16);
  k_vertex<R><<<(unsigned)std::max(1LL, blocks), 32 * warps, smem, ctx().stream>>>(chi, nmat, mstride, estride,
                                                                                     n, S, C, mode, warps, ctx().err);
  count_launch("vertex");
  return fetch_err() == 0;
  }
}

template <typename R> __global__ void k_scale(cx<R>* a, long long n, R s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = s * a[i];
}
template <typename R> void scale_chi(cx<R>* chi, long long n, double s) {
  k_scale<R><<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(chi, n, (R)s);
  count_launch("scale");
}

// ============================================== Matsubara regrid of Sigma ==
// plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182) on the GPU, one thread
// per series (k, a, b): the outermost stored frequency is dropped, the series
// is extended to negative frequencies by Sigma_lm(-iw) = conj Sigma_ml(iw),
// a not-a-knot cubic spline through the n = 2(Nw_old - 1) points of that
// uniform grid (spacing 2 pi T_old) is evaluated at the new frequencies, the
// points beyond the kept cutoff take c0 + c1/(iw) fitted by least squares
// over the stored window [i0, i1) (2x2 normal equations; the Gram matrix is
// the same for every series), and the diagonal is clipped to Im <= 0.  On a
// uniform grid the not-a-knot rows fix M_1 and M_{n-2}; M_2..M_{n-3} solve
// tridiag(1, 4, 1) by the Thomas algorithm with the shared factors cth[].
struct RegridArgs {
  int Nk, Nw_old, Nw_new, No, i0, i1;
  double temp_old, temp_new, w_scale, sw, sw2;  // sum over the window of 1/w and 1/w^2
};

__device__ __forceinline__ double2 regrid_y(const double2* sig, int i, int k, int a, int b, const RegridArgs& r) {
  const int nk = r.Nw_old - 1;
  return i < nk ? conj(sig[fidx(k, nk - 1 - i, b, a, r.Nk, r.Nw_old, r.No)])
                : sig[fidx(k, i - nk, a, b, r.Nk, r.Nw_old, r.No)];
}

__global__ void k_regrid_sigma(double2* out, const double2* sig, double2* dsc, const double* cth, RegridArgs r) {
  const long long NS = (long long)r.Nk * r.No * r.No;
  const int nk = r.Nw_old - 1, n = 2 * nk, m = n - 4;
  const double h = 2.0 * kPi * r.temp_old, h2 = h * h;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < NS;
       s += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(s % r.Nk), a = (int)((s / r.Nk) % r.No), b = (int)(s / ((long long)r.Nk * r.No));
    auto rhs = [&](int i) {  // 6 (y_{i+1} - 2 y_i + y_{i-1}) / h^2
      const double2 d = regrid_y(sig, i + 1, k, a, b, r) - 2.0 * regrid_y(sig, i, k, a, b, r) +
                        regrid_y(sig, i - 1, k, a, b, r);
      return (6.0 / h2) * d;
    };
    const double2 M1 = (1.0 / 6.0) * rhs(1), Mn2 = (1.0 / 6.0) * rhs(n - 2);
    // forward sweep of tridiag(1, 4, 1) for M_2..M_{n-3}, stored [j][series]
    double2 prev = mkc(0.0, 0.0);
    for (int j = 0; j < m; ++j) {
      double2 d = rhs(j + 2);
      if (j == 0) d = d - M1;
      if (j == m - 1) d = d - Mn2;
      d = (j == 0) ? 0.25 * d : (d - prev) * (1.0 / (4.0 - cth[j - 1]));
      dsc[(long long)j * NS + s] = d;
      prev = d;
    }
    for (int j = m - 2; j >= 0; --j) {
      const double2 d = dsc[(long long)j * NS + s] - cth[j] * dsc[(long long)(j + 1) * NS + s];
      dsc[(long long)j * NS + s] = d;
    }
    auto Mat = [&](int i) -> double2 {
      if (i == 1) return M1;
      if (i == n - 2) return Mn2;
      if (i == 0) return 2.0 * M1 - (m > 0 ? dsc[s] : Mn2);
      if (i == n - 1) return 2.0 * Mn2 - (m > 0 ? dsc[(long long)(m - 1) * NS + s] : M1);
      return dsc[(long long)(i - 2) * NS + s];
    };
    // tail c0 + c1/(iw): normal equations of the basis [1, -i/w] over the window
    double2 b0 = mkc(0.0, 0.0), b1 = mkc(0.0, 0.0);
    for (int t = r.i0; t < r.i1; ++t) {
      const double w = (2.0 * t + 1.0) * kPi * r.temp_old;
      const double2 y = sig[fidx(k, t, a, b, r.Nk, r.Nw_old, r.No)];
      b0 += y;
      b1 += mkc(-y.y / w, y.x / w);  // (i/w) y
    }
    const double mw = (double)(r.i1 - r.i0), det = mw * r.sw2 - r.sw * r.sw;
    // G01 = -i sw, G10 = +i sw: c0 = (sw2 b0 + i sw b1)/det, c1 = (-i sw b0 + m b1)/det
    const double2 c0 = (1.0 / det) * (r.sw2 * b0 + mkc(-r.sw * b1.y, r.sw * b1.x));
    const double2 c1 = (1.0 / det) * (mkc(r.sw * b0.y, -r.sw * b0.x) + mw * b1);
    const double x0 = -(2.0 * (nk - 1) + 1.0) * kPi * r.temp_old, xlast = -x0;
    for (int q = 0; q < r.Nw_new; ++q) {
      const double x = r.w_scale * (2.0 * q + 1.0) * kPi * r.temp_new;
      double2 v;
      if (x >= x0 && x <= xlast) {
        int i = (int)floor((x - x0) / h);
        if (i > n - 2) i = n - 2;
        const double xa = x0 + (i + 1) * h - x, xb = x - (x0 + i * h);
        const double2 Mi = Mat(i), Mj = Mat(i + 1);
        const double2 yi = regrid_y(sig, i, k, a, b, r), yj = regrid_y(sig, i + 1, k, a, b, r);
        v = (1.0 / (6.0 * h)) * (xa * xa * xa * Mi + xb * xb * xb * Mj) + xa * ((1.0 / h) * yi - (h / 6.0) * Mi) +
            xb * ((1.0 / h) * yj - (h / 6.0) * Mj);
      } else {
        v = c0 + mkc(c1.y / x, -c1.x / x);  // c1 / (i x)
      }
      if (a == b && v.y > 0) v.y = 0.0;
      out[fidx(k, q, a, b, r.Nk, r.Nw_new, r.No)] = v;
    }
  }
}

void regrid_sigma(double2* out, const double2* sig, int Nk, int Nw_old, int Nw_new, int Norb, double temp_old,
                  double temp_new, double w_scale) {
  PGB_CHECK(Nw_old >= 3, "regrid needs at least 3 stored frequencies");
  PGB_CHECK(Nw_new >= 1 && Nk >= 1 && Norb >= 1, "non-positive regrid size");
  PGB_CHECK(temp_old > 0 && temp_new > 0 && w_scale > 0, "non-positive temperature or frequency scale");
  const int nk = Nw_old - 1, n = 2 * nk, m = n - 4;
  RegridArgs r{Nk, Nw_old, Nw_new, Norb, (int)(0.55 * nk), 0, temp_old, temp_new, w_scale, 0.0, 0.0};
  r.i1 = std::max((int)(0.85 * nk), (int)(0.55 * nk) + 4);
  PGB_CHECK(r.i1 <= nk, "too few stored frequencies for the tail window");
  for (int t = r.i0; t < r.i1; ++t) {
    const double w = (2.0 * t + 1.0) * kPi * temp_old;
    r.sw += 1.0 / w;
    r.sw2 += 1.0 / (w * w);
  }
  std::vector<double> c(std::max(1, m), 0.0);
  if (m > 0) {
    c[0] = 0.25;
    for (int j = 1; j < m; ++j) c[j] = 1.0 / (4.0 - c[j - 1]);
  }
  const long long NS = (long long)Nk * Norb * Norb;
  DBuf<double> dc(c.size());
  dc.upload(c.data(), c.size());
  DBuf<double2> dsc((size_t)std::max(1, m) * NS);
  k_regrid_sigma<<<grid_1d(NS, 128, 65536), 128, 0, ctx().stream>>>(out, sig, dsc.p, dc.p, r);
  count_launch("regrid_sigma");
  sync();
}

// ======================================================= Wannier R space ==
// plibs.output_self_wannier / output_gap_wannier (libs/plibs/_wannier_io.py:
// 52-68, 70-98): data given on the irreducible k points (or on the full grid)
// in the wrappers' layout [Norb][Norb][Nw][Nk] is put on the full grid for
// the first N_cut frequencies, with plain complex conjugation at -k (the
// writers' convention), and inverse-transformed over k with 1/Nkall.  The
// full-grid values go to the positions the spatial backward transform reads
// (FFT4D position tables), so its output is in natural R order.
__global__ void k_wannier_expand(double2* out, const double2* data, const int* grid_irr, const int* grid_flag,
                                 const int* pos_x, const int* pos_y, const int* pos_z, int Nx, int Ny, int Nz,
                                 int Nk, int Nw, int No, int Ncut, int full_bz) {
  const long long Nkall = (long long)Nx * Ny * Nz;
  const long long N = Nkall * Ncut * No * No;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long gi = idx % Nkall;
    const int n = (int)((idx / Nkall) % Ncut);
    const long long e = idx / (Nkall * Ncut);
    const int x = (int)(gi % Nx), y = (int)((gi / Nx) % Ny), z = (int)(gi / ((long long)Nx * Ny));
    const long long p = pos_x[x] + (long long)Nx * (pos_y[y] + (long long)Ny * pos_z[z]);
    double2 v;
    if (full_bz) {
      v = data[(e * Nw + n) * Nkall + gi];
    } else {
      v = data[(e * Nw + n) * Nk + grid_irr[gi]];
      if (grid_flag[gi]) v = conj(v);
    }
    out[(e * Ncut + n) * Nkall + p] = v;
  }
}
__global__ void k_scale64(double2* a, long long n, double s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = s * a[i];
}

void wannier_r(double2* out, const double2* data, const Geom& g, int Nw, int No, int Ncut, bool full_bz) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, Ncut, (int)sizeof(double2));
  const long long N = g.Nkall * Ncut * No * No;
  k_wannier_expand<<<grid_1d(N, 256, 65536), 256, 0, st>>>(out, data, g.grid_irr.p, g.grid_flag.p, fft.d_pos(0),
                                                          fft.d_pos(1), fft.d_pos(2), g.Nx, g.Ny, g.Nz, g.Nk, Nw,
                                                          No, Ncut, full_bz ? 1 : 0);
  count_launch("wannier_expand");
  fft.backward_space<double>(out, No * No, st);
  k_scale64<<<grid_1d(N, 256, 65536), 256, 0, st>>>(out, N, 1.0 / (double)g.Nkall);
  count_launch("scale");
  sync();
}

// ============================================ nonlinear FLEX-Eliashberg ==
// SC Dyson updates of ffeliash.f90:316-377, per (k, iw):
//   G = G0 (I + Delta F^H),   F = -G0 Delta G^H (diagonal real, upper = conj lower)
__global__ void k_mkgreliah(double2* G, const double2* G0, const double2* F, const double2* D, long long K, int No) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    double2 m[kMaxOrb * kMaxOrb];
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 s = mkc(a == b ? 1.0 : 0.0, 0.0);
        for (int c = 0; c < No; ++c) s += D[idx + K * (a + No * c)] * conj(F[idx + K * (b + No * c)]);
        m[a * No + b] = s;
      }
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 s = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) s += G0[idx + K * (a + No * c)] * m[c * No + b];
        G[idx + K * (a + No * b)] = s;
      }
  }
}
__global__ void k_mkfkeliash(double2* F, const double2* G0, const double2* G, const double2* D, long long K, int No) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    double2 m[kMaxOrb * kMaxOrb];
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 s = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) s += D[idx + K * (a + No * c)] * conj(G[idx + K * (b + No * c)]);
        m[a * No + b] = s;
      }
    for (int a = 0; a < No; ++a)
      for (int b = 0; b <= a; ++b) {
        double2 s = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) s += G0[idx + K * (a + No * c)] * m[c * No + b];
        s = -s;
        if (a == b) s.y = 0.0;
        F[idx + K * (a + No * b)] = s;
        if (a != b) F[idx + K * (b + No * a)] = conj(s);
      }
  }
}
void mkgreliah(double2* G, const double2* G0, const double2* F, const double2* D, long long K, int Norb) {
  k_mkgreliah<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(G, G0, F, D, K, Norb);
  count_launch("mkgreliah");
}
void mkfkeliash(double2* F, const double2* G0, const double2* G, const double2* D, long long K, int Norb) {
  k_mkfkeliash<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(F, G0, G, D, K, Norb);
  count_launch("mkfkeliash");
}

// chi^FF padding of one irreducible pair (l, m) (ffeliash.f90:556-570):
// array 2c is F^+14, array 2c+1 is F23; at -k the reference reads
// F(o1[m], o1[l]) for the +iw leg of F^+14 and F(o2[l], o2[m]) for F23.
struct FFPad {
  int o1l, o2l, o1m, o2m;
  double pa, pb;  // prt products times sgn * dprt
};
template <typename R>
__global__ void k_pad_ff(cx<R>* out, const double2* F, const FFPad* pads, const int* grid_irr, const int* grid_flag,
                         long long Nkall, int Nk, int Nw, int No, long long P) {
  const int c = blockIdx.y >> 1, which = blockIdx.y & 1;
  const FFPad t = pads[c];
  cx<R>* o = out + (long long)blockIdx.y * P;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long gi = idx % Nkall;
    const int n = (int)(idx / Nkall);
    const int k = grid_irr[gi], fl = grid_flag[gi];
    double2 v;
    if (n < Nw) {
      if (which == 0) v = conj(fl ? F[fidx(k, n, t.o1m, t.o1l, Nk, Nw, No)] : F[fidx(k, n, t.o2m, t.o1l, Nk, Nw, No)]);
      else v = fl ? F[fidx(k, n, t.o2l, t.o2m, Nk, Nw, No)] : F[fidx(k, n, t.o2l, t.o1m, Nk, Nw, No)];
    } else {
      const int j = 2 * Nw - 1 - n;
      if (which == 0) v = t.pa * conj(F[fidx(k, j, t.o1l, t.o2m, Nk, Nw, No)]);
      else v = t.pb * (fl ? F[fidx(k, j, t.o2l, t.o1m, Nk, Nw, No)] : F[fidx(k, j, t.o1m, t.o2l, Nk, Nw, No)]);
    }
    o[idx] = cmk<R>((R)v.x, (R)v.y);
  }
}

// chi^FF(q, nu) = -sum F^+14(k+q) F23(k) by FFT convolution (ffeliash.f90:491-612)
template <typename R>
void chi0_ff(const Geom& g, const Pairs& p, const double2* F, const std::vector<double>& prt, double temp,
             bool singlet, cx<R>* chi) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, (int)g.M, (int)sizeof(cx<R>));
  const double sgnd = singlet ? 1.0 : 1.0;  // sgn * dprt: (+1)(+1) singlet, (-1)(-1) triplet
  std::vector<FFPad> hp(p.chi.size());
  std::vector<ChiDev> hc(p.chi.size());
  for (size_t i = 0; i < p.chi.size(); ++i) {
    const ChiPair& c = p.chi[i];
    const int o1l = p.o1[c.l], o2l = p.o2[c.l], o1m = p.o1[c.m], o2m = p.o2[c.m];
    hp[i] = FFPad{o1l, o2l, o1m, o2m, prt[o1l] * prt[o2m] * sgnd, prt[o1m] * prt[o2l] * sgnd};
    hc[i] = ChiDev{c.m, c.l, c.m2, c.l2, 0, 0, c.self, 0, make_double2(0, 0), 0, 0, 0, 0, make_double2(0, 0)};
  }
  PGB_CUDA(cudaMemsetAsync(chi, 0, sizeof(cx<R>) * (size_t)g.K * g.Nchi * g.Nchi, st));
  sync();
  const size_t freeb = device_bytes_available();
  long long ch = (long long)((freeb / 4) / (3 * sizeof(cx<R>) * (size_t)g.P));
  ch = std::max(1LL, std::min<long long>(std::min<long long>(ch, 32), (long long)hp.size()));
  DBuf<cx<R>> A((size_t)2 * ch * g.P), T((size_t)ch * g.P);
  DBuf<FFPad> dp(ch);
  DBuf<ChiDev> dc(ch);
  const double sc = temp / (double)g.Nkall / (double)g.P;
  for (long long c0 = 0; c0 < (long long)hp.size(); c0 += ch) {
    const int nc = (int)std::min<long long>(ch, (long long)hp.size() - c0);
    std::vector<ChiDev> cc(hc.begin() + c0, hc.begin() + c0 + nc);
    for (int c = 0; c < nc; ++c) {
      cc[c].e13 = 2 * c;
      cc[c].e42 = 2 * c + 1;
    }
    dp.upload(hp.data() + c0, nc);
    dc.upload(cc.data(), nc);
    k_pad_ff<R><<<dim3(grid_1d(g.P, 256, 4096), 2 * nc), 256, 0, st>>>(A.p, F, dp.p, g.grid_irr.p, g.grid_flag.p,
                                                                      g.Nkall, g.Nk, g.Nw, g.Norb, g.P);
    count_launch("pad_ff");
    fft.forward<R>(A.p, 2 * nc, st);
    k_chi0_product<R><<<mesh_tau_grid(g.Nkall, g.M, nc), 256, 0, st>>>(
        T.p, A.p, nullptr, nullptr, nullptr, dc.p, g.P, g.Nx, g.Ny, g.Nz, (int)g.M, fft.d_rev(0), fft.d_rev(1),
        fft.d_rev(2), fft.d_rev(3), fft.d_logical(3), (R)sc, (R)0);
    count_launch("chi0_product");
    fft.backward<R>(T.p, nc, st);
    k_chi0_scatter<R><<<mesh_tau_grid(g.Nk, g.Nw, nc), 256, 0, st>>>(chi, T.p, dc.p, g.irr_grid.p, nullptr,
                                                                        g.Nkall, g.Nk, g.Nw, g.Nchi, g.P);
    count_launch("chi0_scatter");
    sync();
  }
}

// chi0_S = GG + FF (into gg), chi0_C = GG - FF (into ff)
__global__ void k_combine_sc(double2* gg, double2* ff, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 a = gg[i], b = ff[i];
    gg[i] = a + b;
    ff[i] = a - b;
  }
}
void combine_sc(double2* gg, double2* ff, long long n) {
  k_combine_sc<<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(gg, ff, n);
  count_launch("combine_sc");
}

// V_sigma and V_Delta from chi0_S (in XS) and chi0_C (in XC), in place
// (ffeliash.f90:379-452), one warp per (q, iw), row i on lane i:
//   P = chi0_S S, Q = chi0_C C, chi_s = (I-P)^-1 P, chi_c = (I+Q)^-1 Q,
//   V_sigma = 3/2 S - 1/2 C + 3/2 S chi_s + 1/2 C chi_c - 1/4 (S+C)(P+Q),
//   V_Delta = V0 + cs S chi_s + cc C chi_c  (singlet V0=(S+C)/2, cs=3/2, cc=-1/2;
//             triplet V0=(S-C)/2, cs=cc=-1/2).
// Per warp, shared memory holds P (then chi_s), Q (then chi_c), P+Q (N*N
// each) and an N x 32 accumulation block, one column per lane.
template <int N, int W>
__global__ void __launch_bounds__(32 * W) k_vertex_sc(double2* XS, double2* XC, long long K, const double* S,
                                                      const double* C, int singlet, int* err) {
  extern __shared__ __align__(16) unsigned char smsc[];
  double* sS = reinterpret_cast<double*>(smsc);  // row-major S, C
  double* sC = sS + N * N;
  double2* base = reinterpret_cast<double2*>(smsc + ((2 * N * N * sizeof(double) + 15) / 16) * 16);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int kWarpStride = 3 * N * N + 32 * N;
  double2* Pm = base + (size_t)w * kWarpStride;
  double2* Qm = Pm + N * N;
  double2* X5 = Qm + N * N;
  double2* Rb = X5 + N * N;  // [j][lane], N * 32
  int* ints = reinterpret_cast<int*>(base + (size_t)W * kWarpStride);
  int* pv = ints + w * (N + 1);
  int* mp = ints + W * (N + 1) + w * 32;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    sS[(e % N) * N + e / N] = S[e];  // Fortran (a,b) at a + N b -> row-major
    sC[(e % N) * N + e / N] = C[e];
  }
  __syncthreads();
  const int i = lane < N ? lane : 0;
  const double cs = singlet ? 1.5 : -0.5, cc = -0.5;
  const double v0c = singlet ? 1.0 : -1.0;
  for (long long q = (long long)blockIdx.x * W + w; q < K; q += (long long)gridDim.x * W) {
    double2 a[N];
    // P row i = chi0_S(i,:) S ; Q row i = chi0_C(i,:) C
#pragma unroll
    for (int j = 0; j < N; ++j) a[j] = XS[q + K * (i + N * j)];
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < N; ++c) s += sS[c * N + j] * a[c];
      if (lane < N) Pm[i * N + j] = s;
    }
#pragma unroll
    for (int j = 0; j < N; ++j) a[j] = XC[q + K * (i + N * j)];
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(0.0, 0.0);
#pragma unroll
      for (int c = 0; c < N; ++c) s += sC[c * N + j] * a[c];
      if (lane < N) {
        Qm[i * N + j] = s;
        X5[i * N + j] = Pm[i * N + j] + s;
      }
    }
    __syncwarp();
    bool ok = true;
    for (int pass = 0; pass < 2; ++pass) {
      double2* Mm = pass == 0 ? Pm : Qm;
      const double sg = pass == 0 ? -1.0 : 1.0;  // I - P, I + Q
#pragma unroll
      for (int j = 0; j < N; ++j) a[j] = mkc(i == j ? 1.0 : 0.0, 0.0) + sg * Mm[i * N + j];
      ok &= warp_inverse<double, N>(a, pv, mp);
      for (int j = 0; j < N; ++j) Rb[j * 32 + lane] = mkc(0.0, 0.0);
      for (int c = 0; c < N; ++c) {
        const double2 ac = pick<double, N>(a, c);
        for (int j = 0; j < N; ++j) Rb[j * 32 + lane] += ac * Mm[c * N + j];
      }
      __syncwarp();
      if (lane < N)
        for (int j = 0; j < N; ++j) Mm[i * N + j] = Rb[j * 32 + lane];  // chi_s or chi_c
      __syncwarp();
    }
    if (!ok && lane == 0) atomicExch(err, 5);
    // V_sigma row i
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(1.5 * sS[i * N + j] - 0.5 * sC[i * N + j], 0.0);
      for (int c = 0; c < N; ++c)
        s += 1.5 * sS[i * N + c] * Pm[c * N + j] + 0.5 * sC[i * N + c] * Qm[c * N + j] -
             0.25 * (sS[i * N + c] + sC[i * N + c]) * X5[c * N + j];
      if (lane < N) XS[q + K * (i + N * j)] = s;
    }
    // V_Delta row i
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(0.5 * (sS[i * N + j] + v0c * sC[i * N + j]), 0.0);
      for (int c = 0; c < N; ++c) s += cs * sS[i * N + c] * Pm[c * N + j] + cc * sC[i * N + c] * Qm[c * N + j];
      if (lane < N) XC[q + K * (i + N * j)] = s;
    }
    __syncwarp();
  }
}

bool vertex_sc(double2* XS, double2* XC, long long K, int Nchi, const double* S, const double* C, bool singlet) {
  constexpr int W = 2;
  auto launch = [&](auto kernel, int n) {
    const size_t smem = ((2 * (size_t)n * n * sizeof(double) + 15) / 16) * 16 +
                        (size_t)W * (3 * n * n + 32 * n) * sizeof(double2) + sizeof(int) * (W * (n + 1) + W * 32);
    PGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long blocks = std::min<long long>((K + W - 1) / W, (long long)ctx().num_sms * 16);
    kernel<<<(unsigned)std::max(1LL, blocks), 32 * W, smem, ctx().stream>>>(XS, XC, K, S, C, singlet ? 1 : 0,
                                                                             ctx().err);
  };
  reset_err();
  switch (Nchi) {
    case 1: launch(k_vertex_sc<1, W>, 1); break;
    case 4: launch(k_vertex_sc<4, W>, 4); break;
    case 9: launch(k_vertex_sc<9, W>, 9); break;
    case 16: launch(k_vertex_sc<16, W>, 16); break;
    case 25: launch(k_vertex_sc<25, W>, 25); break;
    default: throw Error("the nonlinear Eliashberg vertex supports Nchi = Norb^2 with Norb <= 5");
  }
  count_launch("vertex_sc");
  return fetch_err() == 0;
}
template void chi0_ff<double>(const Geom&, const Pairs&, const double2*, const std::vector<double>&, double, bool,
                              double2*);

// ====================================================== coarse-mesh seed ==
// Sigma of a coarse mesh on the full coarse grid, [e][n][grid cell], FP32
__global__ void k_sig_to_grid(float2* out, const double2* sig, const int* grid_irr, const int* grid_flag,
                              long long Nkall, int Nk, int Nw, int No) {
  const int e = blockIdx.y, a = e % No, b = e / No;
  const long long N = Nkall * Nw;
  float2* o = out + (long long)e * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long gi = idx % Nkall;
    const int n = (int)(idx / Nkall);
    const int k = grid_irr[gi];
    // Sigma(-k) = Sigma(k)^T under time reversal
    const double2 v = grid_flag[gi] ? sig[fidx(k, n, b, a, Nk, Nw, No)] : sig[fidx(k, n, a, b, Nk, Nw, No)];
    o[idx] = make_float2((float)v.x, (float)v.y);
  }
}

// coarse logical index and weight of fine logical index l along one axis;
// false where the fine Fourier component has no coarse counterpart
__device__ __forceinline__ bool pad_axis(int l, int nc, int nf, int* c, float* w) {
  if (nc == nf) {
    *c = l;
    return true;
  }
  const int r = (l < (nf + 1) / 2) ? l : l - nf;
  const int ar = r < 0 ? -r : r;
  if (nc % 2 == 0) {
    if (ar < nc / 2) {
      *c = (r + nc) % nc;
      return true;
    }
    if (ar == nc / 2) {  // Nyquist plane: half to +nc/2, half to -nc/2
      *c = nc / 2;
      *w *= 0.5f;
      return true;
    }
    return false;
  }
  if (ar <= (nc - 1) / 2) {
    *c = (r + nc) % nc;
    return true;
  }
  return false;
}

struct PadTables {
  int nc[3], nf[3];
  const int* pos_c[3];  // coarse position of each coarse logical index (forward_space layout)
  const int* log_f[3];  // fine logical index of each fine position (backward_space input layout)
};

__global__ void k_pad_space(float2* out, const float2* in, long long Nkc, long long Nkf, int Nw, PadTables t) {
  const int e = blockIdx.y;
  const long long N = Nkf * Nw;
  const float2* src = in + (long long)e * Nkc * Nw;
  float2* o = out + (long long)e * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long s = idx % Nkf, n = idx / Nkf;
    const int p[3] = {(int)(s % t.nf[0]), (int)((s / t.nf[0]) % t.nf[1]), (int)(s / ((long long)t.nf[0] * t.nf[1]))};
    float w = 1.0f;
    int c[3];
    bool in_range = true;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) in_range = in_range && pad_axis(t.log_f[ax][p[ax]], t.nc[ax], t.nf[ax], &c[ax], &w);
    float2 v = make_float2(0.f, 0.f);
    if (in_range) {
      const long long ci = t.pos_c[0][c[0]] + (long long)t.nc[0] * (t.pos_c[1][c[1]] + (long long)t.nc[1] * t.pos_c[2][c[2]]);
      const float2 u = src[n * Nkc + ci];
      v = make_float2(w * u.x, w * u.y);
    }
    o[idx] = v;
  }
}

// fine irreducible Sigma from the interpolated grid; frequencies beyond the
// coarse set from c0 + c1/(i w) through the coarse frequencies n1 < n2
__global__ void k_grid_to_sig(double2* sig, const float2* F, const int* irr_grid, long long Nkall, int Nk, int Nw_c,
                              int Nw_f, int No, double scale, double temp) {
  const long long N = (long long)Nk * Nw_f * No * No;
  const int n2 = Nw_c >= 4 ? Nw_c - 2 : Nw_c - 1;
  const int n1 = Nw_c >= 4 ? (3 * Nw_c) / 4 : n2;
  const double pi = kPi;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk);
    const int n = (int)((idx / Nk) % Nw_f);
    const int e = (int)(idx / ((long long)Nk * Nw_f));
    const float2* base = F + (long long)e * Nkall * Nw_c + irr_grid[k];
    double2 v;
    if (n < Nw_c) {
      const float2 u = base[(long long)n * Nkall];
      v = make_double2(scale * u.x, scale * u.y);
    } else {
      const float2 u1 = base[(long long)n1 * Nkall], u2 = base[(long long)n2 * Nkall];
      const double2 s1 = make_double2(scale * u1.x, scale * u1.y), s2 = make_double2(scale * u2.x, scale * u2.y);
      if (n1 == n2) {
        v = s2;
      } else {
        // z = 1/(i w) = -i/w
        const double2 z1 = make_double2(0.0, -1.0 / ((2 * n1 + 1) * pi * temp));
        const double2 z2 = make_double2(0.0, -1.0 / ((2 * n2 + 1) * pi * temp));
        const double2 zn = make_double2(0.0, -1.0 / ((2 * n + 1) * pi * temp));
        const double2 c1 = cdiv(s1 - s2, z1 - z2);
        const double2 c0 = s1 - c1 * z1;
        v = c0 + c1 * zn;
      }
    }
    sig[idx] = v;
  }
}

void sigma_interp(const Geom& gc, const Geom& gf, const double2* sig_c, double2* sig_f, int No, double temp) {
  cudaStream_t st = ctx().stream;
  PGB_CHECK(gf.Nx % gc.Nx == 0 && gf.Ny % gc.Ny == 0 && gf.Nz % gc.Nz == 0 && gf.Nw >= gc.Nw,
            "coarse mesh does not divide the fine mesh");
  const int No2 = No * No;
  const FFT4D& pc = fft_plan(gc.Nx, gc.Ny, gc.Nz, gc.Nw, (int)sizeof(float2));
  const FFT4D& pf = fft_plan(gf.Nx, gf.Ny, gf.Nz, gc.Nw, (int)sizeof(float2));
  DBuf<float2> A((size_t)No2 * gc.Nkall * gc.Nw), B((size_t)No2 * gf.Nkall * gc.Nw);
  k_sig_to_grid<<<dim3(grid_1d(gc.Nkall * gc.Nw, 256, 4096), No2), 256, 0, st>>>(
      A.p, sig_c, gc.grid_irr.p, gc.grid_flag.p, gc.Nkall, gc.Nk, gc.Nw, No);
  count_launch("sig_to_grid");
  pc.forward_space<float>(A.p, No2, st);
  PadTables t{};
  const int nc[3] = {gc.Nx, gc.Ny, gc.Nz}, nf[3] = {gf.Nx, gf.Ny, gf.Nz};
  for (int ax = 0; ax < 3; ++ax) {
    t.nc[ax] = nc[ax];
    t.nf[ax] = nf[ax];
    t.pos_c[ax] = pc.d_pos(ax);
    t.log_f[ax] = pf.d_logical(ax);
  }
  k_pad_space<<<dim3(grid_1d(gf.Nkall * gc.Nw, 256, 4096), No2), 256, 0, st>>>(B.p, A.p, gc.Nkall, gf.Nkall, gc.Nw,
                                                                                t);
  count_launch("pad_space");
  pf.backward_space<float>(B.p, No2, st);
  const long long N = (long long)gf.Nk * gf.Nw * No2;
  k_grid_to_sig<<<grid_1d(N, 256, 65536), 256, 0, st>>>(sig_f, B.p, gf.irr_grid.p, gf.Nkall, gf.Nk, gc.Nw, gf.Nw, No,
                                                         1.0 / (double)gc.Nkall, temp);
  count_launch("grid_to_sig");
  sync();
}

// ================================================================= sigma ==
template <typename R>
__global__ void k_contract(cx<R>* out, const cx<R>* W, const cx<R>* F, const int* ef, int nt, long long P) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.x * blockDim.x) {
    cx<R> acc = cmk<R>(0, 0);
    for (int t = 0; t < nt; ++t) acc += W[(long long)t * P + idx] * F[(long long)ef[t] * P + idx];
    out[idx] = acc;
  }
}

// All outputs of mkdelta in one launch, from the cached transforms: block x
// is the output (fastest, so the outputs of one index tile run together
// and share the F tiles in L2), blocks y stride over index tiles.  Output o
// sums its terms tb[o] .. tb[o+1]-1 in the order k_contract does:
// T_o = sum_t W_t F_{ef[t]}.
template <typename R>
__global__ void k_contract_all(cx<R>* out, const cx<R>* W, const cx<R>* F, const int* ef, const int* tb,
                               long long P) {
  const int o = blockIdx.x;
  const int t0 = tb[o], t1 = tb[o + 1];
  cx<R>* dst = out + (long long)o * P;
  for (long long idx = (long long)blockIdx.y * blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.y * blockDim.x) {
    cx<R> acc = cmk<R>(0, 0);
    for (int t = t0; t < t1; ++t) acc += W[(long long)t * P + idx] * F[(long long)ef[t] * P + idx];
    dst[idx] = acc;
  }
}

// element type of an untyped work array: 0 float2, 1 double2, 2 double-float
template <typename R> constexpr int elem_kind() { return sizeof(cx<R>) == 8 ? 0 : (sizeof(R) == 8 && sizeof(cx<R>) == 16 && !std::is_same<R, dfl>::value ? 1 : 2); }

__global__ void k_scatter_out(double2* dst, const void* tmp, int kind, const int* irr_grid, long long Nkall,
                              int Nk, int Nw, double scale, int do_thresh) {
  MeshTau q;  // one irreducible k, a chunk of frequencies j
  if (!mesh_tau(Nk, Nw, q)) return;
  const int k = q.r;
  const long long gk = irr_grid[k];
  for (int j = q.t0; j < q.t1; ++j) {
    const long long idx = k + (long long)Nk * j;
    const long long src = gk + Nkall * j;
    double2 v = kind == 1 ? ((const double2*)tmp)[src]
                          : (kind == 0 ? ccast<double>(((const float2*)tmp)[src]) : ccast<double>(((const cdf*)tmp)[src]));
    v = scale * v;
    if (do_thresh) v = thresh(v);
    dst[idx] = v;
  }
}

// Mirror pairs.  The padded bosonic arrays satisfy B_lm(k,s) = conj B_ml(k,-s)
// at every slot except s = 0 (where it needs V(q,0) Hermitian in the pair
// index) and s = Nw (where it needs the static matrix symmetric).  Hence
//   W_lm(r,t) = conj W_ml(-r,t) + D_lm(r) + (-1)^t Nkall [r=0] (stat_lm - stat_ml),
// with D_lm the 3-D transform of d(k) = B_lm(k,0) - conj B_ml(k,0): exact for
// any input, and only Nchi(Nchi+1)/2 forward transforms per stage instead of
// Nchi^2.  One MirrorTerm is a transformed base pair (m,l) (output a+No*b,
// G element ef) and, if mirror != 0, its partner (l,m) (output b+No*a, ef_t).
struct MirrorTerm {
  int m, l, ef, ef_t, mirror, out_t;  // out_t: partner goes to the second output
  double dstat;                        // stat_lm - stat_ml
};

// d(k) of every mirrored term at slot 0 (natural grid order), nt arrays of Nkall
template <typename R>
__global__ void k_mirror_delta0(cx<R>* out, const cx<R>* V, const MirrorTerm* terms, const int* grid_irr,
                                const int* grid_flag, long long Nkall, int Nk, int Nw, int Nchi) {
  const MirrorTerm t = terms[blockIdx.y];
  cx<R>* o = out + (long long)blockIdx.y * Nkall;
  for (long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x; gi < Nkall;
       gi += (long long)gridDim.x * blockDim.x) {
    const int k = grid_irr[gi], fl = grid_flag[gi];
    const cx<R> vlm = V[fidx(k, 0, t.l, t.m, Nk, Nw, Nchi)], vml = V[fidx(k, 0, t.m, t.l, Nk, Nw, Nchi)];
    o[gi] = t.mirror ? (fl ? vml - conj(vlm) : vlm - conj(vml)) : cmk<R>(0, 0);
  }
}

// T0 = sum_t W_t G_ef(t) (+ mirrored partners with out_t == 0),
// T1 = sum of the mirrored partners with out_t == 1.
template <typename R>
__global__ void k_contract_mirror(cx<R>* T0, cx<R>* T1, const cx<R>* W, const cx<R>* F, const cx<R>* D,
                                  const MirrorTerm* terms, int nt, long long P, long long Nkall, int Nx, int Ny,
                                  const int* rev_x, const int* rev_y, const int* rev_z, const int* log_t) {
  __shared__ R s_nk;  // converted once per block (see k_chi0_scatter)
  if (threadIdx.x == 0) s_nk = (R)(double)Nkall;
  __syncthreads();
  const R nk = s_nk;
  MeshTau q;  // one slice per thread: the term loop below already streams many arrays
  if (!mesh_tau(Nkall, P / Nkall, q, 1)) return;
  const int s = q.r;
  const int px = s % Nx, py = (s / Nx) % Ny, pz = s / (Nx * Ny);
  const long long s_m = rev_x[px] + (long long)Nx * (rev_y[py] + (long long)Ny * rev_z[pz]);
  for (int pt = q.t0; pt < q.t1; ++pt) {
    const long long idx = s + Nkall * pt;
    const long long idx_m = s_m + Nkall * pt;
    const R sgn = (log_t[pt] & 1) ? (R)-1 : (R)1;
    cx<R> a0 = cmk<R>(0, 0), a1 = cmk<R>(0, 0);
    for (int i = 0; i < nt; ++i) {
      const MirrorTerm t = terms[i];
      const cx<R>* Wt = W + (long long)i * P;
      a0 += Wt[idx] * F[(long long)t.ef * P + idx];
      if (t.mirror) {
        cx<R> wm = conj(Wt[idx_m]) + D[(long long)i * Nkall + s];
        if (s == 0) wm.x += sgn * nk * (R)t.dstat;
        const cx<R> c = wm * F[(long long)t.ef_t * P + idx];
        if (t.out_t) a1 += c;
        else a0 += c;
      }
    }
    T0[idx] = a0;
    if (T1) T1[idx] = a1;
  }
}

template <typename R>
void sigma(const Geom& g, const Pairs& p, const double2* G, const cx<R>* V, const double* S, const double* C,
           double temp, double2* sig) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, (int)g.M, (int)sizeof(cx<R>));
  const FFT4D& fft3 = fft_plan(g.Nx, g.Ny, g.Nz, 1, (int)sizeof(cx<R>));
  const int No = g.Norb, No2 = No * No, Nchi = g.Nchi;
  DBuf<cx<R>> F((size_t)No2 * g.P);
  pad_green_all<R>(g, G, F.p);
  fft.forward<R>(F.p, No2, st);
  // static slot of V_sigma: 1.5 S - 0.5 C, or S itself when C is null (the
  // spin-orbit loop passes -V there, fselfwithsoc.f90:588)
  std::vector<double> hS(Nchi * Nchi), hC(Nchi * Nchi, 0.0);
  PGB_CUDA(cudaMemcpyAsync(hS.data(), S, sizeof(double) * hS.size(), cudaMemcpyDeviceToHost, st));
  if (C) PGB_CUDA(cudaMemcpyAsync(hC.data(), C, sizeof(double) * hC.size(), cudaMemcpyDeviceToHost, st));
  sync();
  auto stat = [&](int m, int l) {
    return C ? 1.5 * hS[m + Nchi * l] - 0.5 * hC[m + Nchi * l] : hS[m + Nchi * l];
  };
  // groups: output e = a + No*b with a <= b, together with its transpose
  struct Group { int e, et; std::vector<MirrorTerm> terms; };
  std::vector<Group> groups;
  for (int b = 0; b < No; ++b)
    for (int a = 0; a <= b; ++a) {
      Group gr{a + No * b, b + No * a, {}};
      for (const Term& t : p.sigma[gr.e]) {
        if (a == b && t.m > t.l) continue;  // covered as the mirror of (l,m)
        MirrorTerm mt{};
        mt.m = t.m;
        mt.l = t.l;
        mt.ef = t.ef;
        mt.mirror = (t.m != t.l);
        mt.ef_t = p.o2[t.l] + No * p.o2[t.m];
        mt.out_t = (a != b);
        mt.dstat = mt.mirror ? stat(t.l, t.m) - stat(t.m, t.l) : 0.0;
        gr.terms.push_back(mt);
      }
      if (a != b || !gr.terms.empty()) groups.push_back(std::move(gr));
    }
  size_t maxt = 1;
  for (auto& gr : groups) maxt = std::max(maxt, gr.terms.size());
  DBuf<cx<R>> W(maxt * g.P), T((size_t)2 * g.P), Dm(maxt * g.Nkall);
  DBuf<BosonTerm> dterms(maxt);
  DBuf<MirrorTerm> mterms(maxt);
  PGB_CUDA(cudaMemsetAsync(sig, 0, sizeof(double2) * (size_t)g.K * No2, st));
  const double scale = temp / (double)g.Nkall / (double)g.P;
  for (const Group& gr : groups) {
    const int nt = (int)gr.terms.size();
    const bool two = gr.e != gr.et;
    if (nt == 0) continue;
    std::vector<BosonTerm> ht(nt);
    for (int t = 0; t < nt; ++t) ht[t] = BosonTerm{gr.terms[t].m, gr.terms[t].l, stat(gr.terms[t].m, gr.terms[t].l)};
    dterms.upload(ht.data(), nt);
    mterms.upload(gr.terms.data(), nt);
    k_pad_boson<R><<<mesh_tau_grid(g.Nkall, g.M, nt), 256, 0, st>>>(W.p, V, dterms.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw, Nchi,
                                         g.P);
    count_launch("pad_boson");
    fft.forward<R>(W.p, nt, st);
    dim3 grd0(grid_1d(g.Nkall, 256, 4096), nt);
    k_mirror_delta0<R><<<grd0, 256, 0, st>>>(Dm.p, V, mterms.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw,
                                              Nchi);
    count_launch("mirror_delta0");
    fft3.forward<R>(Dm.p, nt, st);
    k_contract_mirror<R><<<mesh_tau_grid(g.Nkall, g.M, 1, 1), 256, 0, st>>>(
        T.p, two ? T.p + g.P : nullptr, W.p, F.p, Dm.p, mterms.p, nt, g.P, g.Nkall, g.Nx, g.Ny, fft.d_rev(0),
        fft.d_rev(1), fft.d_rev(2), fft.d_logical(3));
    count_launch("contract_mirror");
    fft.backward<R>(T.p, two ? 2 : 1, st);
    k_scatter_out<<<mesh_tau_grid(g.Nk, g.Nw, 1), 256, 0, st>>>(sig + (size_t)gr.e * g.K, T.p, elem_kind<R>(),
                                                             g.irr_grid.p, g.Nkall, g.Nk, g.Nw, scale, 1);
    count_launch("scatter_sigma");
    if (two) {
      k_scatter_out<<<mesh_tau_grid(g.Nk, g.Nw, 1), 256, 0, st>>>(sig + (size_t)gr.et * g.K, T.p + g.P, elem_kind<R>(),
                                                               g.irr_grid.p, g.Nkall, g.Nk, g.Nw, scale, 1);
      count_launch("scatter_sigma");
    }
    sync();  // host term buffers are reused by the next group
  }
}

__global__ void k_hf(double2* sig, int Nk, int Nw, int No, int mode, double2* sub) {
  // sub(k,l,m) for m >= l then subtract from every frequency (fself.f90:384-416)
  const long long N = (long long)Nk * No * No;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk);
    const int l = (int)((idx / Nk) % No), m = (int)(idx / ((long long)Nk * No));
    if (m < l) continue;
    double2 v;
    if (mode == 1) {
      v = 0.5 * (sig[fidx(k, 0, l, m, Nk, Nw, No)] + conj(sig[fidx(k, 0, m, l, Nk, Nw, No)]));
    } else {
      double2 s = mkc(0.0, 0.0);
      for (int j = 0; j < Nw; ++j) s += sig[fidx(k, j, l, m, Nk, Nw, No)] + conj(sig[fidx(k, j, m, l, Nk, Nw, No)]);
      v = (0.5 / Nw) * s;
    }
    sub[k + (long long)Nk * (l + No * m)] = v;
    if (l != m) sub[k + (long long)Nk * (m + No * l)] = conj(v);
  }
}
__global__ void k_hf_apply(double2* sig, const double2* sub, int Nk, int Nw, int No) {
  const long long N = (long long)Nk * Nw * No * No;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long k = idx % Nk;
    const long long ab = idx / ((long long)Nk * Nw);
    sig[idx] -= sub[k + Nk * ab];
  }
}
void hf_subtract(double2* sig, int Nk, int Nw, int Norb, int mode) {
  DBuf<double2> sub((size_t)Nk * Norb * Norb);
  k_hf<<<grid_1d((long long)Nk * Norb * Norb, 128, 65536), 128, 0, ctx().stream>>>(sig, Nk, Nw, Norb, mode, sub.p);
  count_launch("hf");
  k_hf_apply<<<grid_1d((long long)Nk * Nw * Norb * Norb, 256, 65536), 256, 0, ctx().stream>>>(sig, sub.p, Nk, Nw, Norb);
  count_launch("hf_apply");
}

// ============================================================ reductions ==
namespace {
constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

__global__ void k_dot_re(double2* part, const double2* a, const double2* b, long long n) {
  __shared__ double red[kRedThreads];
  double acc = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += a[i].x * b[i].x + a[i].y * b[i].y;
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = mkc(red[0], 0.0);
}

__global__ void k_inner_w(double2* part, const double2* a, const double2* b, const double* kw, int Nk, long long n) {
  __shared__ double2 red[kRedThreads];
  double2 acc = mkc(0.0, 0.0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += kw[i % Nk] * (conj(a[i]) * b[i]);
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_sum_parts(double2* out, const double2* part, int n) {
  __shared__ double2 red[kRedThreads];
  double2 acc = mkc(0.0, 0.0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

__global__ void k_filling(double2* part, const double2* eg, const double* eig, int Nk, int Nw, int No, double mu,
                          double temp) {
  __shared__ double2 red[kRedThreads];
  double2 acc = mkc(0.0, 0.0);  // x: self-energy correction sum, y: Fermi sum
  const long long N = (long long)Nk * Nw * No;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int n = (int)(i % No);
    const long long kj = i / No;
    const int k = (int)(kj % Nk), j = (int)(kj / Nk);
    const double2 z = mkc(mu, (2.0 * j + 1.0) * kPi * temp);
    const double e = eig[n + (long long)No * k];
    const double2 t1 = cdiv(mkc(1.0, 0.0), z - eg[n + (long long)No * (k + (long long)Nk * j)]);
    const double2 t2 = cdiv(mkc(1.0, 0.0), z - mkc(e, 0.0));
    acc.x += t1.x - t2.x;
    if (j == 0) acc.y += 0.5 * (1.0 - tanh(0.5 * (e - mu) / temp));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

double2 finish(DBuf<double2>& part, int nparts) {
  DBuf<double2> out(1);
  k_sum_parts<<<1, kRedThreads, 0, ctx().stream>>>(out.p, part.p, nparts);
  count_launch("sum_parts");
  double2 h;
  out.download(&h, 1);
  sync();
  return h;
}
}  // namespace

double dot_re(const double2* a, const double2* b, long long n) {
  DBuf<double2> part(kRedBlocks);
  k_dot_re<<<kRedBlocks, kRedThreads, 0, ctx().stream>>>(part.p, a, b, n);
  count_launch("dot_re");
  return finish(part, kRedBlocks).x;
}

double2 inner_w(const double2* a, const double2* b, const double* kw, int Nk, long long n) {
  DBuf<double2> part(kRedBlocks);
  k_inner_w<<<kRedBlocks, kRedThreads, 0, ctx().stream>>>(part.p, a, b, kw, Nk, n);
  count_launch("inner_w");
  return finish(part, kRedBlocks);
}

double filling(const double2* eig_g, const double* eig, int Nk, int Nw, int Norb, double mu, double temp) {
  DBuf<double2> part(kRedBlocks);
  k_filling<<<kRedBlocks, kRedThreads, 0, ctx().stream>>>(part.p, eig_g, eig, Nk, Nw, Norb, mu, temp);
  count_launch("filling");
  const double2 s = finish(part, kRedBlocks);
  return (s.y + 2.0 * temp * s.x) / (double)Nk;
}

__global__ void k_eig_gkinv(double2* eg, const double2* hamk, const double2* sig, int Nk, int Nw, int No, int* err) {
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk), j = (int)(idx / Nk);
    double2 A[kMaxOrb * kMaxOrb], w[kMaxOrb];
    for (int l = 0; l < No; ++l)
      for (int m = 0; m < No; ++m)
        A[m * No + l] = hamk[m + No * (l + (long long)No * k)] + sig[fidx(k, j, m, l, Nk, Nw, No)];
    if (eigvals_general(A, No, w) < 0) atomicExch(err, 4);
    for (int n = 0; n < No; ++n) eg[n + (long long)No * idx] = w[n];
  }
}

// ---------------------------------------------------- characteristic polynomial
// The filling of get_rn needs, per (k, iw_j), sum_n 1/(z - lambda_n) with
// lambda_n the eigenvalues of H(k) + Sigma(k, iw_j) and z = mu + i w_j
// (fself.f90:662-711).  That sum is p'(z)/p(z) for p(z) = det(z - H - Sigma),
// so the mu search stores the coefficients of p instead of the eigenvalues:
// a Householder reduction to Hessenberg form and the Hessenberg determinant
// recursion p_{m+1} = (z - h_mm) p_m - sum_{i<m} h_im (h_{i+1,i} ... h_{m,m-1}) p_i,
// with no iteration.  Each trial mu then costs one Horner evaluation per (k, j).
// Against the eigenvalue sum, |Re p'/p - sum 1/(z - lambda)| stayed below
// 3e-13 of sum |1/(z - lambda)| over 2e4 random 5-orbital cases with z within
// pi T of the spectrum.
namespace {
template <int N>
__global__ void k_charpoly_gk(double2* cp, const double2* hamk, const double2* sig, int Nk, int Nw) {
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk), j = (int)(idx / Nk);
    double2 A[N][N];
#pragma unroll
    for (int l = 0; l < N; ++l)
#pragma unroll
      for (int m = 0; m < N; ++m)
        A[m][l] = hamk[m + N * (l + (long long)N * k)] + sig[fidx(k, j, m, l, Nk, Nw, N)];
#pragma unroll
    for (int c = 0; c + 2 < N; ++c) {
      double xs = 0;
#pragma unroll
      for (int i = c + 1; i < N; ++i) xs += abs2(A[i][c]);
      const double xn = sqrt(xs);
      if (xn == 0) continue;
      const double2 x0 = A[c + 1][c];
      const double a0 = hypot(x0.x, x0.y);
      const double2 ph = a0 > 0 ? mkc(x0.x / a0, x0.y / a0) : mkc(1.0, 0.0);
      double2 v[N];
      double vn = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        v[i] = (i > c) ? A[i][c] : mkc(0.0, 0.0);
        if (i == c + 1) v[i] = v[i] + mkc(ph.x * xn, ph.y * xn);
        vn += abs2(v[i]);
      }
      if (vn == 0) continue;
      const double sc = 2.0 / vn;
#pragma unroll
      for (int jj = c; jj < N; ++jj) {
        double2 s = mkc(0.0, 0.0);
#pragma unroll
        for (int i = c + 1; i < N; ++i) s += conj(v[i]) * A[i][jj];
        s = sc * s;
#pragma unroll
        for (int i = c + 1; i < N; ++i) A[i][jj] -= v[i] * s;
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        double2 s = mkc(0.0, 0.0);
#pragma unroll
        for (int jj = c + 1; jj < N; ++jj) s += A[i][jj] * v[jj];
        s = sc * s;
#pragma unroll
        for (int jj = c + 1; jj < N; ++jj) A[i][jj] -= s * conj(v[jj]);
      }
#pragma unroll
      for (int i = c + 2; i < N; ++i) A[i][c] = mkc(0.0, 0.0);
    }
    // P[m][d]: coefficient d of p_m (degree m, monic)
    double2 P[N + 1][N + 1];
#pragma unroll
    for (int m = 0; m <= N; ++m)
#pragma unroll
      for (int d = 0; d <= N; ++d) P[m][d] = mkc(0.0, 0.0);
    P[0][0] = mkc(1.0, 0.0);
#pragma unroll
    for (int m = 0; m < N; ++m) {
#pragma unroll
      for (int d = 0; d <= m; ++d) {
        P[m + 1][d + 1] += P[m][d];
        P[m + 1][d] -= A[m][m] * P[m][d];
      }
      double2 prod = mkc(1.0, 0.0);
#pragma unroll
      for (int i = m - 1; i >= 0; --i) {
        prod = prod * A[i + 1][i];
        const double2 f = A[i][m] * prod;
#pragma unroll
        for (int d = 0; d <= i; ++d) P[m + 1][d] -= f * P[i][d];
      }
    }
#pragma unroll
    for (int d = 0; d < N; ++d) cp[d + (long long)N * idx] = P[N][d];
  }
}

template <int N>
__global__ void k_filling_cp(double2* part, const double2* cp, const double* eig, int Nk, int Nw, double mu,
                             double temp) {
  __shared__ double2 red[kRedThreads];
  double2 acc = mkc(0.0, 0.0);  // x: self-energy correction sum, y: Fermi sum
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk), j = (int)(idx / Nk);
    const double w = (2.0 * j + 1.0) * kPi * temp;
    const double2 z = mkc(mu, w);
    double2 p = mkc(1.0, 0.0), dp = mkc(0.0, 0.0);
#pragma unroll
    for (int d = N - 1; d >= 0; --d) {
      dp = dp * z + p;
      p = p * z + cp[d + (long long)N * idx];
    }
    const double2 ip = crecip(p);  // Re(p'/p) with one division
    double s = dp.x * ip.x - dp.y * ip.y;
    // sum_n x_n / (x_n^2 + w^2) with one division: 1/d_n = (prod_{m != n} d_m) / prod_m d_m
    // from prefix and suffix products (each d_n >= w^2 >= (pi T)^2, at most a few hundred)
    double x[N], d[N], pre[N + 1];
    pre[0] = 1.0;
#pragma unroll
    for (int n = 0; n < N; ++n) {
      x[n] = mu - eig[n + (long long)N * k];
      d[n] = fma(x[n], x[n], w * w);
      pre[n + 1] = pre[n] * d[n];
    }
    const double rall = 1.0 / pre[N];
    double suf = 1.0;
#pragma unroll
    for (int n = N - 1; n >= 0; --n) {
      s -= x[n] * (pre[n] * suf * rall);
      suf *= d[n];
      if (j == 0) acc.y += 0.5 * (1.0 - tanh(-0.5 * x[n] / temp));
    }
    acc.x += s;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
}  // namespace

void charpoly_gk(double2* cp, const double2* hamk, const double2* sig, int Nk, int Nw, int Norb) {
  const long long K = (long long)Nk * Nw;
  const unsigned gb = grid_1d(K, 64, 1 << 20);
  switch (Norb) {
#define PGB_CP(n_) case n_: k_charpoly_gk<n_><<<gb, 64, 0, ctx().stream>>>(cp, hamk, sig, Nk, Nw); break;
    PGB_CP(1) PGB_CP(2) PGB_CP(3) PGB_CP(4) PGB_CP(5) PGB_CP(6) PGB_CP(7) PGB_CP(8)
#undef PGB_CP
    default: throw Error("Norb above the engine limit of 8 orbitals");
  }
  count_launch("charpoly_gk");
}

double filling_cp(const double2* cp, const double* eig, int Nk, int Nw, int Norb, double mu, double temp) {
  DBuf<double2> part(kRedBlocks);
  switch (Norb) {
#define PGB_FC(n_) case n_: k_filling_cp<n_><<<kRedBlocks, kRedThreads, 0, ctx().stream>>>(part.p, cp, eig, Nk, Nw, mu, temp); break;
    PGB_FC(1) PGB_FC(2) PGB_FC(3) PGB_FC(4) PGB_FC(5) PGB_FC(6) PGB_FC(7) PGB_FC(8)
#undef PGB_FC
    default: throw Error("Norb above the engine limit of 8 orbitals");
  }
  count_launch("filling_cp");
  const double2 s = finish(part, kRedBlocks);
  return (s.y + 2.0 * temp * s.x) / (double)Nk;
}

bool eig_gkinv(double2* eig_g, const double2* hamk, const double2* sig, int Nk, int Nw, int Norb) {
  reset_err();
  const long long K = (long long)Nk * Nw;
  k_eig_gkinv<<<grid_1d(K, 64, 1 << 20), 64, 0, ctx().stream>>>(eig_g, hamk, sig, Nk, Nw, Norb, ctx().err);
  count_launch("eig_gkinv");
  return fetch_err() == 0;
}

// ============================================================ eliashberg ==
__global__ void k_mkfk(double2* F, const double2* G, const double2* D, long long K, int No) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    double2 g[kMaxOrb * kMaxOrb], d[kMaxOrb * kMaxOrb], t[kMaxOrb * kMaxOrb];
    const long long s = K;
    for (int b = 0; b < No; ++b)
      for (int a = 0; a < No; ++a) {
        g[a * No + b] = G[idx + s * (a + No * b)];
        d[a * No + b] = D[idx + s * (a + No * b)];
      }
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 acc = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) acc += g[a * No + c] * d[c * No + b];
        t[a * No + b] = acc;
      }
    // F = -(G Delta) G^H, then diag real and upper = conj(lower) (feliash.f90:466-481)
    for (int a = 0; a < No; ++a)
      for (int b = 0; b <= a; ++b) {
        double2 acc = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) acc += t[a * No + c] * conj(g[b * No + c]);
        acc = -acc;
        if (a == b) acc.y = 0;
        F[idx + s * (a + No * b)] = acc;
        if (a != b) F[idx + s * (b + No * a)] = conj(acc);
      }
  }
}
void mkfk(double2* F, const double2* G, const double2* D, long long K, int Norb) {
  k_mkfk<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(F, G, D, K, Norb);
  count_launch("mkfk");
}

// F = -(G Delta) G^H in double-float for the double-float Eliashberg stage:
// G already in double-float, Delta (the FP64 Arnoldi vector) converted once
// per element; the products run on the FP32 pipe instead of the FP64 one
template <int N>
__global__ void k_mkfk_df(cdf* F, const cdf* G, const double2* D, long long K) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    cdf d[N * N];
#pragma unroll
    for (int b = 0; b < N; ++b)
#pragma unroll
      for (int a = 0; a < N; ++a) {
        const double2 v = D[idx + K * (a + N * b)];
        d[a * N + b] = mkc(dfl(v.x), dfl(v.y));
      }
#pragma unroll 1
    for (int a = 0; a < N; ++a) {
      cdf t[N];
#pragma unroll
      for (int b = 0; b < N; ++b) {
        cdf acc = mkc(dfl(0.f), dfl(0.f));
#pragma unroll
        for (int c = 0; c < N; ++c) acc += G[idx + K * (a + N * c)] * d[c * N + b];
        t[b] = acc;
      }
      for (int b = 0; b <= a; ++b) {
        cdf acc = mkc(dfl(0.f), dfl(0.f));
#pragma unroll
        for (int c = 0; c < N; ++c) acc += t[c] * conj(G[idx + K * (b + N * c)]);
        acc = -acc;
        if (a == b) acc.y = dfl(0.f);
        F[idx + K * (a + N * b)] = acc;
        if (a != b) F[idx + K * (b + N * a)] = conj(acc);
      }
    }
  }
}

// false: no double-float kernel for this orbital count (the caller uses mkfk)
bool mkfk_df(cdf* F, const cdf* G, const double2* D, long long K, int Norb) {
  const unsigned grid = grid_1d(K, 128, 65536);
  switch (Norb) {
    case 1: k_mkfk_df<1><<<grid, 128, 0, ctx().stream>>>(F, G, D, K); break;
    case 2: k_mkfk_df<2><<<grid, 128, 0, ctx().stream>>>(F, G, D, K); break;
    case 3: k_mkfk_df<3><<<grid, 128, 0, ctx().stream>>>(F, G, D, K); break;
    case 4: k_mkfk_df<4><<<grid, 128, 0, ctx().stream>>>(F, G, D, K); break;
    case 5: k_mkfk_df<5><<<grid, 128, 0, ctx().stream>>>(F, G, D, K); break;
    default: return false;
  }
  count_launch("mkfk_df");
  return true;
}

__global__ void k_hermitize(double2* D, long long K, int No) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    for (int l = 0; l < No; ++l) {
      D[idx + K * (l + No * l)].y = 0;
      for (int m = l + 1; m < No; ++m) D[idx + K * (l + No * m)] = conj(D[idx + K * (m + No * l)]);
    }
  }
}
void hermitize(double2* D, long long K, int Norb) {
  k_hermitize<<<grid_1d(K, 256, 65536), 256, 0, ctx().stream>>>(D, K, Norb);
  count_launch("hermitize");
}

template <typename R>
void mkdelta(const Geom& g, const Pairs& p, const double2* F, const cx<R>* Vd, const double* S, const double* C,
             const double* prt, bool singlet, double scale, double2* out, DeltaKernelCache<R>* cache,
             const cx<R>* Fbulk) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, (int)g.M, (int)sizeof(cx<R>));
  const int No2 = g.Norb * g.Norb;
  const double sgn = singlet ? 1.0 : -1.0, dprt = singlet ? 1.0 : -1.0;
  DBuf<cx<R>> FF((size_t)No2 * g.P);
  if (Fbulk) {
    k_pad_anomalous_bulk<R><<<mesh_tau_grid(g.Nkall, g.M, No2), 256, 0, st>>>(
        FF.p, Fbulk, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw, g.Norb, g.P, prt, sgn, dprt);
  } else {
    k_pad_anomalous<R><<<mesh_tau_grid(g.Nkall, g.M, No2), 256, 0, st>>>(
        FF.p, F, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw, g.Norb, g.P, prt, sgn, dprt);
  }
  count_launch("pad_anomalous");
  fft.forward<R>(FF.p, No2, st);
  std::vector<double> hS(g.Nchi * g.Nchi), hC(g.Nchi * g.Nchi);
  PGB_CUDA(cudaMemcpyAsync(hS.data(), S, sizeof(double) * hS.size(), cudaMemcpyDeviceToHost, st));
  PGB_CUDA(cudaMemcpyAsync(hC.data(), C, sizeof(double) * hC.size(), cudaMemcpyDeviceToHost, st));
  sync();
  size_t maxt = 0, total = 0;
  for (auto& v : p.delta) { maxt = std::max(maxt, v.size()); total += v.size(); }
  auto terms_of = [&](int e, std::vector<BosonTerm>& ht, std::vector<int>& hef) {
    const auto& terms = p.delta[e];
    ht.resize(terms.size());
    hef.resize(terms.size());
    for (size_t t = 0; t < terms.size(); ++t) {
      const int m = terms[t].m, l = terms[t].l;
      ht[t] = BosonTerm{m, l, 0.5 * (hS[m + g.Nchi * l] + sgn * hC[m + g.Nchi * l])};
      hef[t] = terms[t].ef;
    }
  };
  DBuf<BosonTerm> dterms(std::max<size_t>(1, maxt));
  DBuf<int> def(std::max<size_t>(1, maxt));
  // cache the transformed pairing vertex across Arnoldi steps when it fits
  if (cache && !cache->built) {
    sync();
    const size_t freeb = device_bytes_available();
    const size_t need = total * (size_t)g.P * sizeof(cx<R>);
    cache->built = true;
    if (need < freeb * 0.7) {
      cache->W.alloc(total * (size_t)g.P);
      cache->offset.assign(No2, 0);
      long long off = 0;
      for (int e = 0; e < No2; ++e) {
        cache->offset[e] = off;
        if (p.delta[e].empty()) continue;
        std::vector<BosonTerm> ht;
        std::vector<int> hef;
        terms_of(e, ht, hef);
        dterms.upload(ht.data(), ht.size());
        k_pad_boson<R><<<mesh_tau_grid(g.Nkall, g.M, (unsigned)ht.size()), 256, 0, st>>>(cache->W.p + off * g.P, Vd, dterms.p, g.grid_irr.p, g.grid_flag.p,
                                            g.Nkall, g.Nk, g.Nw, g.Nchi, g.P);
        count_launch("pad_vdelta");
        fft.forward<R>(cache->W.p + off * g.P, (int)ht.size(), st);
        sync();
        off += (long long)ht.size();
      }
    }
  }
  const bool use_cache = cache && cache->W.p;
  PGB_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)g.K * No2, st));
  if (use_cache) {
    // every output in one contraction launch and one batched backward
    // transform, when their transforms fit beside the cache
    if (cache->out_elems.empty()) {
      std::vector<int> hef, htb(1, 0);
      for (int e = 0; e < No2; ++e) {
        if (p.delta[e].empty()) continue;
        std::vector<BosonTerm> ht;
        std::vector<int> he;
        terms_of(e, ht, he);
        hef.insert(hef.end(), he.begin(), he.end());
        htb.push_back((int)hef.size());
        cache->out_elems.push_back(e);
      }
      cache->ef.alloc(std::max<size_t>(1, hef.size()));
      cache->ef.upload(hef.data(), hef.size());
      cache->tb.alloc(htb.size());
      cache->tb.upload(htb.data(), htb.size());
      sync();
    }
    const int ne = (int)cache->out_elems.size();
    if (ne > 0 && (size_t)ne * g.P * sizeof(cx<R>) < device_bytes_available() * 0.7) {
      DBuf<cx<R>> TA((size_t)ne * g.P);
      const unsigned tiles = (unsigned)std::min<long long>((g.P + 255) / 256, 65535);
      k_contract_all<R><<<dim3((unsigned)ne, tiles), 256, 0, st>>>(TA.p, cache->W.p, FF.p, cache->ef.p,
                                                                  cache->tb.p, g.P);
      count_launch("contract_all");
      fft.backward<R>(TA.p, ne, st);
      for (int o = 0; o < ne; ++o) {
        const int e = cache->out_elems[o];
        k_scatter_out<<<mesh_tau_grid(g.Nk, g.Nw, 1), 256, 0, st>>>(out + (size_t)e * g.K, TA.p + (size_t)o * g.P,
                                                                   elem_kind<R>(), g.irr_grid.p, g.Nkall, g.Nk,
                                                                   g.Nw, scale, 0);
        count_launch("scatter_delta");
      }
      sync();
      hermitize(out, g.K, g.Norb);
      return;
    }
  }
  DBuf<cx<R>> W, T(g.P);
  if (!use_cache) W.alloc(std::max<size_t>(1, maxt) * g.P);
  for (int e = 0; e < No2; ++e) {
    if (p.delta[e].empty()) continue;
    std::vector<BosonTerm> ht;
    std::vector<int> hef;
    terms_of(e, ht, hef);
    const int nt = (int)ht.size();
    def.upload(hef.data(), nt);
    const cx<R>* Wp;
    if (use_cache) {
      Wp = cache->W.p + cache->offset[e] * g.P;
    } else {
      dterms.upload(ht.data(), nt);
      k_pad_boson<R><<<mesh_tau_grid(g.Nkall, g.M, nt), 256, 0, st>>>(W.p, Vd, dterms.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw,
                                          g.Nchi, g.P);
      count_launch("pad_vdelta");
      fft.forward<R>(W.p, nt, st);
      Wp = W.p;
    }
    k_contract<R><<<grid_1d(g.P, 256, 65536), 256, 0, st>>>(T.p, Wp, FF.p, def.p, nt, g.P);
    count_launch("contract");
    fft.backward<R>(T.p, 1, st);
    k_scatter_out<<<mesh_tau_grid(g.Nk, g.Nw, 1), 256, 0, st>>>(out + (size_t)e * g.K, T.p, elem_kind<R>(), g.irr_grid.p,
                                                             g.Nkall, g.Nk, g.Nw, scale, 0);
    count_launch("scatter_delta");
    sync();
  }
  hermitize(out, g.K, g.Norb);
}

__global__ void k_initial_delta(double2* D, const double* init, const double2* uni, int Nk, int Nw, int No,
                                int gap_sym) {
  const long long K = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx % Nk);
    if (gap_sym == 0) {
      for (int b = 0; b < No; ++b)
        for (int a = 0; a < No; ++a) D[idx + K * (a + No * b)] = mkc(a == b ? 1.0 : 0.0, 0.0);
      continue;
    }
    const double2* U = uni + (long long)No * No * k;
    // delta0 = U diag(init) U^H, lower triangle then Hermitian (feliash.f90:685-699)
    for (int a = 0; a < No; ++a)
      for (int b = 0; b <= a; ++b) {
        double2 acc = mkc(0.0, 0.0);
        for (int n = 0; n < No; ++n) acc += (init[k + (long long)Nk * n] * U[a + No * n]) * conj(U[b + No * n]);
        if (a == b) acc.y = 0;
        D[idx + K * (a + No * b)] = acc;
        if (a != b) D[idx + K * (b + No * a)] = conj(acc);
      }
  }
}
void initial_delta(double2* D, const double* init, const double2* uni, int Nk, int Nw, int Norb, int gap_sym) {
  const long long K = (long long)Nk * Nw;
  k_initial_delta<<<grid_1d(K, 128, 65536), 128, 0, ctx().stream>>>(D, init, uni, Nk, Nw, Norb, gap_sym);
  count_launch("initial_delta");
}

__global__ void k_axpy(double2* y, double2 a, const double2* x, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void k_scal(double2* y, double a, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = a * y[i];
}
struct LinComb {
  const double2* x[64];
  double2 c[64];
};
__global__ void k_lincomb(double2* y, LinComb lc, int m, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 acc = mkc(0.0, 0.0);
    for (int t = 0; t < m; ++t) acc += lc.c[t] * lc.x[t][i];
    y[i] = acc;
  }
}
void axpy(double2* y, double2 a, const double2* x, long long n) {
  k_axpy<<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(y, a, x, n);
  count_launch("axpy");
}
void scal(double2* y, double a, long long n) {
  k_scal<<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(y, a, n);
  count_launch("scal");
}
void lincomb(double2* y, const double2* const* xs, const double2* cs, int m, long long n) {
  PGB_CHECK(m <= 64, "linear combination of more than 64 vectors");
  LinComb lc{};
  for (int i = 0; i < m; ++i) { lc.x[i] = xs[i]; lc.c[i] = cs[i]; }
  k_lincomb<<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(y, lc, m, n);
  count_launch("lincomb");
}

template <typename R> __global__ void k_widen(double2* out, const cx<R>* in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = ccast<double>(in[i]);
}
template <typename R> __global__ void k_narrow(cx<R>* out, const double2* in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = cmk<R>((R)in[i].x, (R)in[i].y);
}
template <typename R> void widen(double2* out, const cx<R>* in, long long n) {
  k_widen<R><<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(out, in, n);
  count_launch("widen");
}
template <typename R> void narrow(cx<R>* out, const double2* in, long long n) {
  k_narrow<R><<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(out, in, n);
  count_launch("narrow");
}

// conversions between bulk types (double-float <-> float without the FP64 pipe)
__device__ __forceinline__ void cvt(float2& o, float2 v) { o = v; }
__device__ __forceinline__ void cvt(double2& o, double2 v) { o = v; }
__device__ __forceinline__ void cvt(cdf& o, cdf v) { o = v; }
__device__ __forceinline__ void cvt(float2& o, double2 v) { o = make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ void cvt(double2& o, float2 v) { o = make_double2(v.x, v.y); }
__device__ __forceinline__ void cvt(cdf& o, float2 v) { o = mkc(dfl(v.x), dfl(v.y)); }
__device__ __forceinline__ void cvt(float2& o, cdf v) { o = make_float2(v.x.hi + v.x.lo, v.y.hi + v.y.lo); }
__device__ __forceinline__ void cvt(cdf& o, double2 v) { o = mkc(dfl(v.x), dfl(v.y)); }
__device__ __forceinline__ void cvt(double2& o, cdf v) { o = make_double2((double)v.x, (double)v.y); }
template <typename To, typename From>
__global__ void k_convert(cx<To>* out, const cx<From>* in, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    cvt(out[i], in[i]);
}
template <typename To, typename From> void convert(cx<To>* out, const cx<From>* in, long long n) {
  k_convert<To, From><<<grid_1d(n, 256, 65536), 256, 0, ctx().stream>>>(out, in, n);
  count_launch("convert");
}
template void convert<float, dfl>(float2*, const cdf*, long long);
template void convert<dfl, float>(cdf*, const float2*, long long);
template void convert<double, dfl>(double2*, const cdf*, long long);
template void convert<dfl, double>(cdf*, const double2*, long long);
template void convert<float, double>(float2*, const double2*, long long);
template void convert<double, float>(double2*, const float2*, long long);

// ======================================================== instantiations ==
#define PGB_INST(R)                                                                                        \
  template void chi0<R>(const Geom&, const Pairs&, const double2*, double, const TailRef*, cx<R>*);        \
  template void stoner<R>(const Geom&, const cx<R>*, const double*, const double*, double*, double*, int*, \
                          int*);                                                                           \
  template bool vertex<R>(cx<R>*, long long, long long, int, const double*, const double*, int);          \
  template void scale_chi<R>(cx<R>*, long long, double);                                                   \
  template void sigma<R>(const Geom&, const Pairs&, const double2*, const cx<R>*, const double*,           \
                         const double*, double, double2*);                                                 \
  template void mkdelta<R>(const Geom&, const Pairs&, const double2*, const cx<R>*, const double*,         \
                           const double*, const double*, bool, double, double2*, DeltaKernelCache<R>*,     \
                           const cx<R>*);                                                                  \
  template void widen<R>(double2*, const cx<R>*, long long);                                               \
  template void narrow<R>(cx<R>*, const double2*, long long);
PGB_INST(float)
PGB_INST(double)
// double-float bulk: the FFT convolution stages and the conversions around them
template void chi0<dfl>(const Geom&, const Pairs&, const double2*, double, const TailRef*, cx<dfl>*);
template void stoner<dfl>(const Geom&, const cx<dfl>*, const double*, const double*, double*, double*, int*, int*);
template void scale_chi<dfl>(cx<dfl>*, long long, double);
template void sigma<dfl>(const Geom&, const Pairs&, const double2*, const cx<dfl>*, const double*, const double*,
                         double, double2*);
template void widen<dfl>(double2*, const cx<dfl>*, long long);
template void narrow<dfl>(cx<dfl>*, const double2*, long long);
template void mkdelta<dfl>(const Geom&, const Pairs&, const double2*, const cx<dfl>*, const double*, const double*,
                           const double*, bool, double, double2*, DeltaKernelCache<dfl>*, const cx<dfl>*);
template bool vertex<dfl>(cx<dfl>*, long long, long long, int, const double*, const double*, int);

}  // namespace pgb

// ================================================== spin-orbit coupling ==
// fchi0withsoc.f90, fselfwithsoc.f90, feliashwithsoc.f90, fUJ.f90:367-399.
// The chi0 and Sigma stages run through chi0 / sigma above with the spin map
// of Geom; this section holds the parts that differ in kind: the RPA vertex
// -V (I + chi0 V)^-1, the nu = 0 channel sums, and the Eliashberg pieces,
// whose gap lives on the full k mesh in the reference's full-list order.
namespace pgb {

void build_full_mesh(FullMesh& fm, const Geom& g, const int64_t* invk) {
  const long long n = g.Nkall;
  std::vector<int> irr(n), flag(n), minus(n), grid(n, -1);
  for (long long i = 0; i < n; ++i) {
    irr[i] = (int)invk[3 * i] - 1;
    flag[i] = (int)invk[3 * i + 1];
    minus[i] = (int)invk[3 * i + 2] - 1;
    PGB_CHECK(minus[i] >= 0 && minus[i] < n, "invk(3,:) outside [1,Nkall]");
  }
  for (long long gi = 0; gi < n; ++gi) grid[g.h_full_of_grid[gi]] = (int)gi;
  fm.Nkall = n;
  fm.irr.alloc(n);
  fm.irr.upload(irr.data(), n);
  fm.flag.alloc(n);
  fm.flag.upload(flag.data(), n);
  fm.minus.alloc(n);
  fm.minus.upload(minus.data(), n);
  fm.grid.alloc(n);
  fm.grid.upload(grid.data(), n);
  fm.full.alloc(n);
  fm.full.upload(g.h_full_of_grid.data(), n);
}

namespace {
// V_sigma / V_Delta = -V + V (I + X V)^-1 X V = -V (I + X V)^-1 per (q, iw),
// in place; one warp per matrix, row i on lane i (fUJ.f90:367-399)
template <int N, int W>
__global__ void __launch_bounds__(32 * W) k_vertex_soc(double2* chi, long long K, const double* V, int* err) {
  extern __shared__ __align__(16) unsigned char smv[];
  double* sV = reinterpret_cast<double*>(smv);  // row-major V
  double2* base = reinterpret_cast<double2*>(smv + ((N * N * sizeof(double) + 15) / 16) * 16);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double2* Ai = base + (size_t)w * N * N;
  int* ints = reinterpret_cast<int*>(base + (size_t)W * N * N);
  int* pv = ints + w * (N + 1);
  int* mp = ints + W * (N + 1) + w * 32;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) sV[(e % N) * N + e / N] = V[e];
  __syncthreads();
  const int i = lane < N ? lane : 0;
  for (long long q = (long long)blockIdx.x * W + w; q < K; q += (long long)gridDim.x * W) {
    double2 x[N], a[N];
#pragma unroll
    for (int j = 0; j < N; ++j) x[j] = chi[q + K * (i + N * j)];
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(i == j ? 1.0 : 0.0, 0.0);
#pragma unroll
      for (int c = 0; c < N; ++c) s += sV[c * N + j] * x[c];
      a[j] = s;
    }
    const bool ok = warp_inverse<double, N>(a, pv, mp);
    if (lane < N)
      for (int j = 0; j < N; ++j) Ai[i * N + j] = a[j];
    __syncwarp();
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(0.0, 0.0);
      for (int c = 0; c < N; ++c) s += sV[i * N + c] * Ai[c * N + j];
      if (lane < N) chi[q + K * (i + N * j)] = -s;
    }
    __syncwarp();
    if (!ok && lane == 0) atomicExch(err, 6);
  }
}

// Y = (I + chi0(q,0) V)^-1 chi0(q,0) per irreducible q (fchi0withsoc.f90:297-304)
template <int N, int W>
__global__ void __launch_bounds__(32 * W) k_rpa0_soc(double2* Y, const double2* chi, int Nk, long long K,
                                                     const double* V, int* err) {
  extern __shared__ __align__(16) unsigned char smr[];
  double* sV = reinterpret_cast<double*>(smr);
  int* ints = reinterpret_cast<int*>(smr + ((N * N * sizeof(double) + 15) / 16) * 16);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* pv = ints + w * (N + 1);
  int* mp = ints + W * (N + 1) + w * 32;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) sV[(e % N) * N + e / N] = V[e];
  __syncthreads();
  const int i = lane < N ? lane : 0;
  for (int q = blockIdx.x * W + w; q < Nk; q += gridDim.x * W) {
    double2 x[N], a[N];
#pragma unroll
    for (int j = 0; j < N; ++j) x[j] = chi[q + K * (i + N * j)];
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(i == j ? 1.0 : 0.0, 0.0);
#pragma unroll
      for (int c = 0; c < N; ++c) s += sV[c * N + j] * x[c];
      a[j] = s;
    }
    const bool ok = warp_inverse<double, N>(a, pv, mp);
    for (int j = 0; j < N; ++j) {
      double2 s = mkc(0.0, 0.0);
      for (int c = 0; c < N; ++c) s += pick<double, N>(a, c) * chi[q + K * (c + N * j)];
      if (lane < N) Y[q + (long long)Nk * (i + N * j)] = s;
    }
    if (!ok && lane == 0) atomicExch(err, 7);
  }
}

struct ChanTerm {
  int m, l;
  double coef;
};
// out[c][q] = sum of coef * Y(q, m, l) over the terms of output cell c
__global__ void k_chan_sum(double2* out, const double2* Y, const int* start, const ChanTerm* terms, int Nk, int ncell,
                           int N) {
  const long long n = (long long)Nk * ncell;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(idx % Nk), c = (int)(idx / Nk);
    double2 s = mkc(0.0, 0.0);
    for (int t = start[c]; t < start[c + 1]; ++t) s += terms[t].coef * Y[q + (long long)Nk * (terms[t].m + N * terms[t].l)];
    out[idx] = s;
  }
}

// F = -G(k) Delta(k) G(-k)^H on the full mesh, G(-k) from the spin-orbit TRS
// partner, then the spin-block fills of feliashwithsoc.f90:466-516
__global__ void k_mkfk_soc(double2* F, const double2* G, const double2* D, const int* irr, const int* flag,
                           long long Nkall, int Nk, int Nw, int No, SpinMap sm, int gap_sym) {
  const long long n = Nkall * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % Nkall;
    const int j = (int)(idx / Nkall);
    const int k = irr[i], fl = flag[i];
    auto g1 = [&](int a, int c) {  // G(k)_{ac}
      return fl ? (double)(sm.sgn[a] * sm.sgn[c]) * G[fidx(k, j, sm.inv[c], sm.inv[a], Nk, Nw, No)]
                : G[fidx(k, j, a, c, Nk, Nw, No)];
    };
    auto g2 = [&](int b, int c) {  // G(-k)_{bc}
      return fl ? G[fidx(k, j, c, b, Nk, Nw, No)]
                : (double)(sm.sgn[b] * sm.sgn[c]) * G[fidx(k, j, sm.inv[b], sm.inv[c], Nk, Nw, No)];
    };
    double2 Cm[kMaxOrb * kMaxOrb], Fm[kMaxOrb * kMaxOrb];
    for (int a = 0; a < No; ++a)
      for (int c = 0; c < No; ++c) {
        double2 s = mkc(0.0, 0.0);
        for (int e = 0; e < No; ++e) s += g1(a, e) * D[fidx(i, j, e, c, Nkall, Nw, No)];
        Cm[a * kMaxOrb + c] = s;
      }
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 s = mkc(0.0, 0.0);
        for (int c = 0; c < No; ++c) s += Cm[a * kMaxOrb + c] * conj(g2(b, c));
        Fm[a * kMaxOrb + b] = -s;
      }
    auto f = [&](int a, int b) -> double2& { return Fm[a * kMaxOrb + b]; };
    for (int l = 0; l < No; ++l) {
      if (sm.sgn[l] != 1) continue;
      for (int m = 0; m < No; ++m) {
        if (sm.sgn[m] == 1) {
          if (gap_sym < 0) {
            f(sm.inv[l], sm.inv[m]) = -conj(f(m, l));
          } else {
            f(m, l) = mkc(0.0, 0.0);
            f(sm.inv[l], sm.inv[m]) = mkc(0.0, 0.0);
          }
        } else if (sm.inv[m] == l) {
          f(sm.inv[l], sm.inv[m]) = mkc(f(m, l).x, 0.0);
        }
      }
    }
    if (gap_sym != -10)
      for (int l = 0; l < No; ++l) {
        if (sm.sgn[l] != 1) continue;
        for (int m = 0; m < No; ++m)
          if (sm.sgn[m] == -1) f(sm.inv[m], sm.inv[l]) = gap_sym < 0 ? f(m, l) : -f(m, l);
      }
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) F[fidx(i, j, a, b, Nkall, Nw, No)] = Fm[a * kMaxOrb + b];
  }
}

// padded full-mesh F element (a, b): slot j = F(k, iw_j), slot 2Nw-1-j = -F_ba(-k, iw_j)
// (feliashwithsoc.f90:594-601)
__global__ void k_pad_ffull(double2* out, const double2* F, const int* full_of_grid, const int* minus,
                            long long Nkall, int Nw, int No, long long P) {
  const int e = blockIdx.y, a = e % No, b = e / No;
  double2* o = out + (long long)e * P;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long gi = idx % Nkall;
    const int n = (int)(idx / Nkall);
    const int i = full_of_grid[gi];
    o[idx] = n < Nw ? F[fidx(i, n, a, b, Nkall, Nw, No)] : -F[fidx(minus[i], 2 * Nw - 1 - n, b, a, Nkall, Nw, No)];
  }
}

struct SocBoson {
  int m, l, ism, isl;
  double stat, sg2;
};
// pairing-vertex pad of mkdelta_soc: at -q the spin-flipped pair times
// sgnsig2(m,l); slot Nw = -V(m,l) (feliashwithsoc.f90:548-574)
__global__ void k_pad_boson_socd(double2* out, const double2* V, const SocBoson* terms, const int* grid_irr,
                                 const int* grid_flag, long long Nkall, int Nk, int Nw, int Nchi, long long P) {
  const SocBoson t = terms[blockIdx.y];
  double2* o = out + (long long)blockIdx.y * P;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long gi = idx % Nkall;
    const int n = (int)(idx / Nkall);
    const int k = grid_irr[gi], fl = grid_flag[gi];
    double2 v;
    if (n == Nw) {
      v = mkc(t.stat, 0.0);
    } else if (n < Nw) {
      v = fl ? t.sg2 * V[fidx(k, n, t.isl, t.ism, Nk, Nw, Nchi)] : V[fidx(k, n, t.m, t.l, Nk, Nw, Nchi)];
    } else {
      const int j = 2 * Nw - n;
      v = fl ? t.sg2 * conj(V[fidx(k, j, t.ism, t.isl, Nk, Nw, Nchi)]) : conj(V[fidx(k, j, t.l, t.m, Nk, Nw, Nchi)]);
    }
    o[idx] = v;
  }
}

// T = sum_t W_t * FP_{ef_t}
__global__ void k_prodsum(double2* T, const double2* W, const double2* FP, const int* ef, int nt, long long P) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < P;
       idx += (long long)gridDim.x * blockDim.x) {
    double2 s = mkc(0.0, 0.0);
    for (int t = 0; t < nt; ++t) s += W[(long long)t * P + idx] * FP[(long long)ef[t] * P + idx];
    T[idx] = s;
  }
}

// D(i, j) = scale * T(cell of i, j), every full k
__global__ void k_scatter_full(double2* D, const double2* T, const int* grid_of_full, long long Nkall, int Nw,
                               double scale) {
  const long long n = Nkall * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % Nkall, j = idx / Nkall;
    D[idx] = scale * T[grid_of_full[i] + Nkall * j];
  }
}

// spin-block fills of mkdelta_soc (feliashwithsoc.f90:622-662), per (k, iw)
__global__ void k_sym_delta_soc(double2* D, long long Nkall, int Nw, int No, SpinMap sm, int gap_sym) {
  const long long n = Nkall * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx % Nkall;
    const int j = (int)(idx / Nkall);
    auto d = [&](int a, int b) -> double2& { return D[fidx(i, j, a, b, Nkall, Nw, No)]; };
    for (int l = 0; l < No; ++l) {
      if (sm.sgn[l] != 1) continue;
      for (int m = 0; m < No; ++m) {
        if (sm.sgn[m] == 1) d(sm.inv[l], sm.inv[m]) = -conj(d(m, l));
        else if (sm.inv[m] == l) d(l, m) = mkc(d(l, m).x, 0.0);
        else if (l > sm.inv[m]) d(sm.inv[m], sm.inv[l]) = conj(d(l, m));
      }
    }
    if (gap_sym == -10) continue;
    for (int l = 0; l < No; ++l) {
      if (sm.sgn[l] != 1) continue;
      for (int m = 0; m < No; ++m)
        if (sm.sgn[m] == -1) d(sm.inv[l], sm.inv[m]) = gap_sym > 0 ? -d(l, m) : d(l, m);
    }
  }
}

// band gap phi_n(k) to the orbital basis on the full mesh (feliashwithsoc.f90:690-725)
__global__ void k_init_delta_soc(double2* D, const double* init, const double2* uni, const int* irr, const int* flag,
                                 long long Nkall, int Nk, int Nw, int No, SpinMap sm, int gap_sym) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nkall;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = irr[i], fl = flag[i];
    auto U = [&](int a, int n) { return uni[a + (long long)No * (n + (long long)No * k)]; };
    for (int a = 0; a < No; ++a)
      for (int b = 0; b < No; ++b) {
        double2 s = mkc(0.0, 0.0);
        for (int n = 0; n < No; ++n) {
          const double ph = init[k + (long long)Nk * n];
          if (fl == 0) s += (ph * (double)sm.sgn[b]) * (U(a, n) * conj(U(sm.inv[b], n)));
          else s += (ph * (double)sm.sgn[a]) * (conj(U(sm.inv[a], n)) * U(b, n));
        }
        if (fl == 0) s = -s;
        if (gap_sym > 0 && sm.sgn[a] * sm.sgn[b] >= 0) s = mkc(0.0, 0.0);
        for (int j = 0; j < Nw; ++j) D[fidx(i, j, a, b, Nkall, Nw, No)] = s;
      }
  }
}

// orbital gap at the first frequency to the band basis (feliashwithsoc.f90:750-794)
__global__ void k_orb_to_band_soc(double2* out, const double2* D, const double2* uni, const int* irr,
                                  const int* flag, long long Nkall, int Nw, int No, SpinMap sm) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Nkall;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = irr[i], fl = flag[i];
    auto U = [&](int a, int n) { return uni[a + (long long)No * (n + (long long)No * k)]; };
    for (int x = 0; x < No; ++x)
      for (int y = 0; y < No; ++y) {
        double2 s = mkc(0.0, 0.0);
        for (int a = 0; a < No; ++a)
          for (int b = 0; b < No; ++b) {
            const double2 d = D[fidx(i, 0, a, b, Nkall, Nw, No)];
            if (fl == 0) s += (double)sm.sgn[b] * (conj(U(a, x)) * d * U(sm.inv[b], y));
            else s += (double)(-sm.sgn[a]) * (U(sm.inv[a], x) * d * conj(U(b, y)));
          }
        out[i + Nkall * (x + (long long)No * y)] = (fl == 0 || fl == 1) ? s : mkc(0.0, 0.0);
      }
  }
}
}  // namespace

bool vertex_soc(double2* chi, long long K, int Nchi, const double* V) {
  constexpr int W = 4;
  auto launch = [&](auto kernel, int n) {
    const size_t smem = ((size_t)n * n * sizeof(double) + 15) / 16 * 16 + (size_t)W * n * n * sizeof(double2) +
                        sizeof(int) * (W * (n + 1) + W * 32);
    PGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long blocks = std::min<long long>((K + W - 1) / W, (long long)ctx().num_sms * 16);
    kernel<<<(unsigned)std::max(1LL, blocks), 32 * W, smem, ctx().stream>>>(chi, K, V, ctx().err);
  };
  reset_err();
  switch (Nchi) {
    case 4: launch(k_vertex_soc<4, W>, 4); break;
    case 16: launch(k_vertex_soc<16, W>, 16); break;
    default: throw Error("the spin-orbit vertex supports Nchi = 4 or 16 (2 or 4 spin-orbitals)");
  }
  count_launch("vertex_soc");
  return fetch_err() == 0;
}

void chis_chic_soc(double2* chic, double2* chiszz, double2* chispm, const double2* chi, long long K, int Nk, int Nchi,
                   const double* V, const std::vector<int>& o1, const std::vector<int>& o2,
                   const std::vector<int>& slist, const std::vector<int>& orb_list) {
  constexpr int W = 4;
  const int n4 = Nchi / 4;
  DBuf<double2> Y((size_t)Nk * Nchi * Nchi);
  auto launch = [&](auto kernel, int n) {
    const size_t smem = ((size_t)n * n * sizeof(double) + 15) / 16 * 16 + sizeof(int) * (W * (n + 1) + W * 32);
    const long long blocks = std::min<long long>((Nk + W - 1) / W, (long long)ctx().num_sms * 16);
    kernel<<<(unsigned)std::max(1LL, blocks), 32 * W, smem, ctx().stream>>>(Y.p, chi, Nk, K, V, ctx().err);
  };
  reset_err();
  switch (Nchi) {
    case 4: launch(k_rpa0_soc<4, W>, 4); break;
    case 16: launch(k_rpa0_soc<16, W>, 16); break;
    default: throw Error("get_chis_chic_soc supports Nchi = 4 or 16 (2 or 4 spin-orbitals)");
  }
  count_launch("rpa0_soc");
  PGB_CHECK(fetch_err() == 0, "zgesv failed in get_chis_chic_soc");
  // output cells: channel c (0 chic, 1 chiszz, 2 chispm) x (r, s); the reference
  // accumulates cmat2(m,l) into cell (orb_list(l), orb_list(m)) by spin labels
  const int ncell = 3 * n4 * n4;
  std::vector<std::vector<ChanTerm>> cell(ncell);
  auto s = [&](int a) { return slist[a]; };
  for (int l = 0; l < Nchi; ++l)
    for (int m = 0; m < Nchi; ++m) {
      const int r = orb_list[l] - 1, c = orb_list[m] - 1;
      PGB_CHECK(r >= 0 && r < n4 && c >= 0 && c < n4, "orb_list entry outside [1,Nchi/4]");
      const int rc = r + n4 * c;
      if (s(o1[l]) == s(o1[m]) && s(o2[l]) == s(o2[m]) && s(o1[l]) == -s(o2[l]) && s(o1[l]) == 1)
        cell[2 * n4 * n4 + rc].push_back({m, l, 1.0});
      if (s(o1[l]) == s(o2[l]) && s(o1[m]) == s(o2[m])) {
        cell[rc].push_back({m, l, 0.5});
        cell[n4 * n4 + rc].push_back({m, l, s(o1[l]) == s(o1[m]) ? 0.25 : -0.25});
      }
    }
  std::vector<int> start(ncell + 1, 0);
  std::vector<ChanTerm> flat;
  for (int c = 0; c < ncell; ++c) {
    start[c] = (int)flat.size();
    flat.insert(flat.end(), cell[c].begin(), cell[c].end());
  }
  start[ncell] = (int)flat.size();
  DBuf<int> dstart(ncell + 1);
  dstart.upload(start.data(), ncell + 1);
  DBuf<ChanTerm> dterms(std::max<size_t>(1, flat.size()));
  if (!flat.empty()) dterms.upload(flat.data(), flat.size());
  DBuf<double2> out((size_t)Nk * ncell);
  k_chan_sum<<<grid_1d((long long)Nk * ncell, 256, 65536), 256, 0, ctx().stream>>>(out.p, Y.p, dstart.p, dterms.p,
                                                                                   Nk, ncell, Nchi);
  count_launch("chan_sum");
  const size_t cs = (size_t)Nk * n4 * n4;
  out.download(chic, cs);
  PGB_CUDA(cudaMemcpyAsync(chiszz, out.p + cs, cs * sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream));
  PGB_CUDA(cudaMemcpyAsync(chispm, out.p + 2 * cs, cs * sizeof(double2), cudaMemcpyDeviceToHost, ctx().stream));
  sync();
}

void mkfk_soc(double2* F, const double2* G, const double2* D, const FullMesh& fm, const Geom& g, int gap_sym) {
  const long long n = fm.Nkall * g.Nw;
  k_mkfk_soc<<<grid_1d(n, 128, 65536), 128, 0, ctx().stream>>>(F, G, D, fm.irr.p, fm.flag.p, fm.Nkall, g.Nk, g.Nw,
                                                               g.Norb, g.spin, gap_sym);
  count_launch("mkfk_soc");
}

void mkdelta_soc(const Geom& g, const Pairs& p, const FullMesh& fm, const double2* F, const double2* Vd,
                 const std::vector<double>& Vmat, const std::vector<int>& invschi, int gap_sym, double scale,
                 double2* out) {
  cudaStream_t st = ctx().stream;
  const FFT4D& fft = fft_plan(g.Nx, g.Ny, g.Nz, (int)g.M, (int)sizeof(double2));
  const int No = g.Norb, No2 = No * No, Nchi = g.Nchi;
  const long long KF = fm.Nkall * g.Nw;
  const int* s = g.spin.sgn;
  const int* inv = g.spin.inv;
  // terms grouped by output element (o1 l, o2 m) (feliashwithsoc.f90:538-545)
  std::vector<std::vector<std::pair<SocBoson, int>>> groups(No2);
  for (int l = 0; l < Nchi; ++l)
    for (int m = 0; m < Nchi; ++m) {
      const int o1l = p.o1[l], o2l = p.o2[l], o1m = p.o1[m], o2m = p.o2[m];
      const bool mixed = s[o1l] * s[o2m] < 0;
      if (!(gap_sym < 0 || (gap_sym > 0 && mixed))) continue;
      if (!((gap_sym == -10 && mixed) || s[o1l] == 1)) continue;
      if (!(s[o2m] == 1 || o1l >= inv[o2m])) continue;
      const double sg2 = (double)(s[o1m] * s[o2m] * s[o1l] * s[o2l]);
      PGB_CHECK(invschi[l] >= 1 && invschi[m] >= 1 && invschi[l] <= Nchi && invschi[m] <= Nchi,
                "invschi entry outside [1,Nchi] (olist lacks a spin-flipped pair)");
      SocBoson t{m, l, invschi[m] - 1, invschi[l] - 1, -Vmat[m + (size_t)Nchi * l], sg2};
      groups[o1l + No * o2m].push_back({t, o2l + No * o1m});
    }
  DBuf<double2> FP((size_t)No2 * g.P);
  dim3 gp(grid_1d(g.P, 256, 4096), No2);
  k_pad_ffull<<<gp, 256, 0, st>>>(FP.p, F, fm.full.p, fm.minus.p, fm.Nkall, g.Nw, No, g.P);
  count_launch("pad_ffull");
  fft.forward<double>(FP.p, No2, st);
  size_t maxt = 1;
  for (auto& gr : groups) maxt = std::max(maxt, gr.size());
  DBuf<double2> W(maxt * g.P), T(g.P);
  DBuf<SocBoson> dt(maxt);
  DBuf<int> def(maxt);
  PGB_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)KF * No2, st));
  for (int e = 0; e < No2; ++e) {
    const int nt = (int)groups[e].size();
    if (nt == 0) continue;
    std::vector<SocBoson> ht(nt);
    std::vector<int> hef(nt);
    for (int t = 0; t < nt; ++t) {
      ht[t] = groups[e][t].first;
      hef[t] = groups[e][t].second;
    }
    dt.upload(ht.data(), nt);
    def.upload(hef.data(), nt);
    dim3 gw(grid_1d(g.P, 256, 4096), nt);
    k_pad_boson_socd<<<gw, 256, 0, st>>>(W.p, Vd, dt.p, g.grid_irr.p, g.grid_flag.p, g.Nkall, g.Nk, g.Nw, Nchi, g.P);
    count_launch("pad_boson_socd");
    fft.forward<double>(W.p, nt, st);
    k_prodsum<<<grid_1d(g.P, 256, 65536), 256, 0, st>>>(T.p, W.p, FP.p, def.p, nt, g.P);
    count_launch("prodsum");
    fft.backward<double>(T.p, 1, st);
    k_scatter_full<<<grid_1d(KF, 256, 65536), 256, 0, st>>>(out + (size_t)e * KF, T.p, fm.grid.p, fm.Nkall, g.Nw,
                                                            scale / (double)g.P);
    count_launch("scatter_full");
    sync();  // host term buffers are reused by the next element
  }
  k_sym_delta_soc<<<grid_1d(KF, 128, 65536), 128, 0, st>>>(out, fm.Nkall, g.Nw, No, g.spin, gap_sym);
  count_launch("sym_delta_soc");
}

void initial_delta_soc(double2* D, const double* init, const double2* uni, const FullMesh& fm, const Geom& g,
                       int gap_sym) {
  k_init_delta_soc<<<grid_1d(fm.Nkall, 128, 65536), 128, 0, ctx().stream>>>(D, init, uni, fm.irr.p, fm.flag.p,
                                                                             fm.Nkall, g.Nk, g.Nw, g.Norb, g.spin,
                                                                             gap_sym);
  count_launch("init_delta_soc");
}

void orb_to_band_soc(double2* out, const double2* D, const double2* uni, const FullMesh& fm, const Geom& g) {
  k_orb_to_band_soc<<<grid_1d(fm.Nkall, 128, 65536), 128, 0, ctx().stream>>>(out, D, uni, fm.irr.p, fm.flag.p,
                                                                              fm.Nkall, g.Nw, g.Norb, g.spin);
  count_launch("orb_to_band_soc");
}
}  // namespace pgb

// ======================================================= real frequency ==
// Band-basis Lindhard sums on the real axis (fchi.f90:95-318, fphi.f90:89-305)
// and Pade continuation (fpade.f90).  The reference adds rank-1 terms
// w_klm B B^T (N^6 per k); here chi_{ab,cd} = sum_k sum_lm P_ac,l(k+q) w_lm
// Q_bd,m(k) is contracted as (P W) Q^T (N^5 per k) in shared memory, one
// CTA per (q, w) job and one thread per output element.
namespace pgb {
namespace {
template <int PHI>
__global__ void k_bubble_rf(double2* out, const double2* uni, const double* eig, const double* ff, const int* qsh,
                            const RfJob* jobs, const int* o1, const int* o2, int Nk, int No, int Nchi, double mu,
                            double temp, double eps) {
  extern __shared__ __align__(16) unsigned char smb[];
  const int N2 = No * No, N3 = N2 * No;
  double2* Uk = reinterpret_cast<double2*>(smb);  // [a + No n]
  double2* Uq = Uk + N2;
  double2* W = Uq + N2;   // [l + No m]
  double2* P = W + N2;    // [(a + No c) + N2 l]
  double2* Q = P + N3;    // [(b + No d) + N2 m]
  double2* T = Q + N3;    // [(a + No c) + N2 m]
  double* e_k = reinterpret_cast<double*>(T + N3);
  double* e_q = e_k + No;
  double* f_k = e_q + No;
  double* f_q = f_k + No;
  const RfJob jb = jobs[blockIdx.x];
  const int* qs = qsh + jb.qoff;
  const int t = threadIdx.x, nt = blockDim.x;
  const bool active = t < Nchi * Nchi;
  const int i = t % Nchi, j = t / Nchi;
  const int ac = active ? o1[i] + No * o1[j] : 0, bd = active ? o2[i] + No * o2[j] : 0;
  const double temp_safe = fmax(temp, 1.0e-12);
  double2 acc = mkc(0.0, 0.0);
  for (int k = 0; k < Nk; ++k) {
    const int kq = qs[k];
    for (int e = t; e < N2; e += nt) {
      Uk[e] = uni[e + (long long)N2 * k];
      Uq[e] = uni[e + (long long)N2 * kq];
    }
    for (int e = t; e < No; e += nt) {
      e_k[e] = eig[e + (long long)No * k];
      e_q[e] = eig[e + (long long)No * kq];
      f_k[e] = ff[e + (long long)No * k];
      f_q[e] = ff[e + (long long)No * kq];
    }
    __syncthreads();
    for (int e = t; e < N2; e += nt) {  // weight of band pair (l at k+q, m at k)
      const int l = e % No, m = e / No;
      double2 w = mkc(0.0, 0.0);
      if (PHI) {
        const double den = jb.w - e_k[m] - e_q[l] + 2.0 * mu;
        if (!(fabs(den) < eps && jb.delta < eps)) w = cdiv(mkc(-(1.0 - f_q[l] - f_k[m]), 0.0), mkc(den, jb.delta));
      } else {
        const double de = e_k[m] - e_q[l];
        if (fabs(jb.w) < 1.0e-12 && fabs(de) < 1.0e-9) w = mkc(f_k[m] * (1.0 - f_k[m]) / temp_safe, 0.0);
        else if (fabs(f_q[l] - f_k[m]) > eps) w = cdiv(mkc(f_q[l] - f_k[m], 0.0), mkc(jb.w + de, jb.delta));
      }
      W[e] = w;
    }
    for (int e = t; e < N3; e += nt) {
      const int pr = e % N2, n = e / N2, a = pr % No, c = pr / No;
      P[e] = conj(Uq[a + No * n]) * Uq[c + No * n];
      Q[e] = Uk[a + No * n] * conj(Uk[c + No * n]);
    }
    __syncthreads();
    for (int e = t; e < N3; e += nt) {
      const int pr = e % N2, m = e / N2;
      double2 s = mkc(0.0, 0.0);
      for (int l = 0; l < No; ++l) s += P[pr + N2 * l] * W[l + No * m];
      T[e] = s;
    }
    __syncthreads();
    if (active)
      for (int m = 0; m < No; ++m) acc += T[ac + N2 * m] * Q[bd + N2 * m];
    __syncthreads();
  }
  if (active) out[i + (long long)Nchi * (j + (long long)Nchi * blockIdx.x)] = (1.0 / (double)Nk) * acc;
}

// chi_s = (I - chi0 S)^-1 chi0 per q and the (ll, mm) sums of chi_s and chi0
// (fchi.f90:289-314); one warp per q
template <int N>
__global__ void k_rpa_trace(double2* trs, double2* tr0, const double2* chi, const double* S, const int* dmask,
                            int Nq, int* err) {
  __shared__ int piv[4][N + 1], map[4][32];
  __shared__ double sS[N * N];
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) sS[(e % N) * N + e / N] = S[e];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = lane < N ? lane : 0;
  for (int q = blockIdx.x * 4 + w; q < Nq; q += gridDim.x * 4) {
    const double2* X = chi + (long long)N * N * q;  // X(i, j) at i + N j
    double2 a[N];
    for (int jj = 0; jj < N; ++jj) {
      double2 s = mkc(i == jj ? 1.0 : 0.0, 0.0);
      for (int c = 0; c < N; ++c) s -= sS[c * N + jj] * X[i + N * c];
      a[jj] = s;
    }
    const bool ok = warp_inverse<double, N>(a, piv[w], map[w]);
    double2 s_s = mkc(0.0, 0.0), s_0 = mkc(0.0, 0.0);
    if (lane < N && dmask[i])
      for (int jj = 0; jj < N; ++jj) {
        if (!dmask[jj]) continue;
        double2 v = mkc(0.0, 0.0);
        for (int c = 0; c < N; ++c) v += pick<double, N>(a, c) * X[c + N * jj];
        s_s += v;
        s_0 += X[i + N * jj];
      }
    for (int off = 16; off > 0; off >>= 1) {
      s_s.x += __shfl_xor_sync(0xffffffffu, s_s.x, off);
      s_s.y += __shfl_xor_sync(0xffffffffu, s_s.y, off);
      s_0.x += __shfl_xor_sync(0xffffffffu, s_0.x, off);
      s_0.y += __shfl_xor_sync(0xffffffffu, s_0.y, off);
    }
    if (lane == 0) {
      trs[q] = s_s;
      tr0[q] = s_0;
      if (!ok) atomicExch(err, 8);
    }
  }
}

__global__ void k_trace_jobs(double2* tr, const double2* m, int N, int Nq) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Nq; q += gridDim.x * blockDim.x) {
    double2 s = mkc(0.0, 0.0);
    for (int l = 0; l < N; ++l) s += m[l + (long long)N * (l + (long long)N * q)];
    tr[q] = s;
  }
}

// Pade: coefficients of series (k, o) = A(k, :, o, o) (fpade.f90:1-27); only the
// entries j >= i of g_i are formed, the ones later steps read
__global__ void k_pade_coef(double2* a, double2* g, const double2* A, const double2* xn, int Nk, int Np, int No) {
  const long long ns = (long long)Nk * No;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ns; s += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(s % Nk), o = (int)(s / Nk);
    double2* gs = g + s * Np;
    double2* as = a + s * Np;
    for (int jj = 0; jj < Np; ++jj) gs[jj] = A[k + (long long)Nk * (jj + (long long)Np * (o + (long long)No * o))];
    as[0] = gs[0];
    for (int ii = 1; ii < Np; ++ii) {
      const double2 gp = gs[ii - 1], xp = xn[ii - 1];
      for (int jj = ii; jj < Np; ++jj) {
        const double2 gj = gs[jj];
        gs[jj] = (gj.x == 0.0 && gj.y == 0.0) ? mkc(0.0, 0.0) : cdiv(gp - gj, (xn[jj] - xp) * gj);
      }
      as[ii] = gs[ii];
    }
  }
}

// out(w, k) = sum_o P_N / Q_N of series (k, o) at wl(w) (fpade.f90:29-129)
__global__ void k_pade_eval(double2* out, const double2* a, const double2* xn, const double2* wl, int Nk, int Np,
                            int Nw, int No) {
  const long long n = (long long)Nk * Nw;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int w = (int)(idx % Nw), k = (int)(idx / Nw);
    const double2 z = wl[w];
    double2 sum = mkc(0.0, 0.0);
    for (int o = 0; o < No; ++o) {
      const double2* as = a + ((long long)k + (long long)Nk * o) * Np;
      double2 P0 = mkc(0.0, 0.0), P1 = as[0], Q0 = mkc(1.0, 0.0), Q1 = mkc(1.0, 0.0);
      for (int ii = 1; ii < Np; ++ii) {
        const double2 tt = as[ii] * (z - xn[ii - 1]);
        const double2 P = P1 + tt * P0, Q = Q1 + tt * Q0;
        P0 = P1;
        P1 = P;
        Q0 = Q1;
        Q1 = Q;
      }
      sum += cdiv(P1, Q1);
    }
    out[w + (long long)Nw * k] = sum;
  }
}
}  // namespace

void bubble_rf(double2* out, const double2* uni, const double* eig, const double* ff, const int* qsh,
               const std::vector<RfJob>& jobs, const std::vector<int>& o1, const std::vector<int>& o2, int Nk, int No,
               int Nchi, double mu, double temp, double eps, bool phi) {
  PGB_CHECK(No <= kMaxOrb && Nchi <= kMaxChi, "Norb or Nchi above the engine limits");
  DBuf<RfJob> dj(jobs.size());
  dj.upload(jobs.data(), jobs.size());
  DBuf<int> d1(Nchi), d2(Nchi);
  d1.upload(o1.data(), Nchi);
  d2.upload(o2.data(), Nchi);
  const int threads = std::max(32, ((Nchi * Nchi + 31) / 32) * 32);
  const size_t smem = (3 * (size_t)No * No + 3 * (size_t)No * No * No) * sizeof(double2) + 4 * (size_t)No * sizeof(double);
  const long long nj = (long long)jobs.size();
  for (long long j0 = 0; j0 < nj; j0 += 65535) {  // grid.x stays within one launch's limit
    const int nb = (int)std::min<long long>(65535, nj - j0);
    if (phi)
      k_bubble_rf<1><<<nb, threads, smem, ctx().stream>>>(out + (size_t)Nchi * Nchi * j0, uni, eig, ff, qsh, dj.p + j0,
                                                         d1.p, d2.p, Nk, No, Nchi, mu, temp, eps);
    else
      k_bubble_rf<0><<<nb, threads, smem, ctx().stream>>>(out + (size_t)Nchi * Nchi * j0, uni, eig, ff, qsh, dj.p + j0,
                                                         d1.p, d2.p, Nk, No, Nchi, mu, temp, eps);
    count_launch(phi ? "bubble_rf_phi" : "bubble_rf");
  }
}

void rpa_trace(double2* trs, double2* tr0, const double2* chi, const double* S, const int* dmask, int Nchi, int Nq) {
  reset_err();
  const unsigned blocks = (unsigned)std::min<long long>((Nq + 3) / 4, 65535LL);
  switch (Nchi) {
    case 1: k_rpa_trace<1><<<blocks, 128, 0, ctx().stream>>>(trs, tr0, chi, S, dmask, Nq, ctx().err); break;
    case 4: k_rpa_trace<4><<<blocks, 128, 0, ctx().stream>>>(trs, tr0, chi, S, dmask, Nq, ctx().err); break;
    case 9: k_rpa_trace<9><<<blocks, 128, 0, ctx().stream>>>(trs, tr0, chi, S, dmask, Nq, ctx().err); break;
    case 16: k_rpa_trace<16><<<blocks, 128, 0, ctx().stream>>>(trs, tr0, chi, S, dmask, Nq, ctx().err); break;
    case 25: k_rpa_trace<25><<<blocks, 128, 0, ctx().stream>>>(trs, tr0, chi, S, dmask, Nq, ctx().err); break;
    default: throw Error("chiq_map supports Nchi = Norb^2 with Norb <= 5");
  }
  count_launch("rpa_trace");
  PGB_CHECK(fetch_err() == 0, "zgesv failed in chiq_map");
}

void trace_jobs(double2* tr, const double2* m, int Nchi, int Nq) {
  k_trace_jobs<<<grid_1d(Nq, 128, 65536), 128, 0, ctx().stream>>>(tr, m, Nchi, Nq);
  count_launch("trace_jobs");
}

void pade_trace(double2* out, const double2* A, const double2* xn, const double2* wl, int Nk, int Np, int Nw, int No) {
  const long long ns = (long long)Nk * No;
  DBuf<double2> a((size_t)ns * Np), g((size_t)ns * Np);
  k_pade_coef<<<grid_1d(ns, 64, 65536), 64, 0, ctx().stream>>>(a.p, g.p, A, xn, Nk, Np, No);
  count_launch("pade_coef");
  k_pade_eval<<<grid_1d((long long)Nk * Nw, 128, 65536), 128, 0, ctx().stream>>>(out, a.p, xn, wl, Nk, Np, Nw, No);
  count_launch("pade_eval");
}
}  // namespace pgb
