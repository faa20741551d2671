// FLEX self-consistency loop and linearized-Eliashberg solver on the GPU.
//
// Host code here only orchestrates: every array operation is a kernel of
// flex.cu; the host keeps the scalar control flow of the reference (DIIS
// coefficient solve of a (m+1)^2 system, the Brent/bisection search for mu,
// the m x m Hessenberg eigenproblem of Arnoldi), all in FP64.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <fstream>
#include <memory>
#include <vector>

#include "drivers.cuh"
#include "linalg.cuh"

namespace pgb {

namespace {

// the statistics of the last solve called from this thread
thread_local LastStats g_stats;

struct Timer {
  cudaEvent_t a, b;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  void start() { cudaEventRecord(a, ctx().stream); }
  double stop() {
    cudaEventRecord(b, ctx().stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
};

__global__ void k_sub(double2* out, const double2* a, const double2* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = a[i] - b[i];
}

struct DiisTerms {
  const double2* x[16];
  double c[16];
};

// sigma_diis = sum c_i x_i; relative change estimate; mixing (fself.f90:494-532)
__global__ void k_diis_mix(double2* sig, const double2* sig0, DiisTerms t, int n, double pp, int use_diis,
                           double* partmax, long long N) {
  __shared__ double red[256];
  double mx = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    double2 sd = mkc(0.0, 0.0);
    for (int h = 0; h < n; ++h) sd += t.c[h] * t.x[h][i];
    const double2 s0 = sig0[i];
    const double asd = hypot(sd.x, sd.y);
    if (asd > 1.0e-10) {
      const double2 d = s0 - sd;
      mx = fmax(mx, hypot(d.x, d.y) / asd);
    }
    sig[i] = use_diis ? sd : (pp * sd + (1.0 - pp) * s0);
  }
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partmax[blockIdx.x] = red[0];
}

__global__ void k_max_parts(double* out, const double* part, int n) {
  __shared__ double red[256];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, part[i]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// real (n x n) solve with partial pivoting; false if singular (dgesv semantics)
bool solve_real(std::vector<double> A, std::vector<double>& b, int n) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > std::fabs(A[p * n + k])) p = i;
    if (A[p * n + k] == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < n; ++i) {
      const double l = A[i * n + k] / A[k * n + k];
      for (int j = k; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
      b[i] -= l * b[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    double s = b[k];
    for (int j = k + 1; j < n; ++j) s -= A[k * n + j] * b[j];
    b[k] = s / A[k * n + k];
  }
  return true;
}

// ----------------------------------------------------------- sigma.bin --
// gfortran sequential unformatted records (4-byte length markers), written
// and read like io_sigma / ck_sigma_meta (fself.f90:742-780).
void write_record(std::ofstream& f, const void* data, size_t bytes) {
  PGB_CHECK(bytes < 2147483639ULL, "sigma.bin record above 2 GiB is not supported");
  const int32_t n = (int32_t)bytes;
  f.write((const char*)&n, 4);
  f.write((const char*)data, (std::streamsize)bytes);
  f.write((const char*)&n, 4);
}
bool read_record(std::ifstream& f, void* data, size_t bytes) {
  int32_t n = 0, m = 0;
  if (!f.read((char*)&n, 4)) return false;
  if ((size_t)n != bytes) throw Error("sigma.bin record of " + std::to_string(n) + " bytes, expected " +
                                      std::to_string(bytes));
  f.read((char*)data, (std::streamsize)bytes);
  f.read((char*)&m, 4);
  PGB_CHECK(f && m == n, "sigma.bin record markers do not match");
  return true;
}

void write_sigma_bin(double mu, double mu_old, const std::vector<double2>& sig, double temp, int Nw, int Norb,
                     int Nk) {
  std::ofstream f("sigma.bin", std::ios::binary | std::ios::trunc);
  PGB_CHECK(f.good(), "cannot open sigma.bin for writing");
  write_record(f, &mu, 8);
  write_record(f, &mu_old, 8);
  write_record(f, sig.data(), sig.size() * sizeof(double2));
  const double meta[4] = {temp, (double)Nw, (double)Norb, (double)Nk};
  write_record(f, meta, sizeof(meta));
}

// a seed of the FLEX loop must be finite: NaN or Inf would run the loop to
// its iteration cap on a NaN residual
void require_finite(const double2* v, size_t n, const char* what) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i].x) || !std::isfinite(v[i].y))
      throw BadInput(std::string(what) + " holds NaN or Inf (element " + std::to_string(i) + ")");
}

void read_sigma_bin(double& mu, double& mu_old, std::vector<double2>& sig, double temp, int Nw, int Norb, int Nk) {
  std::ifstream f("sigma.bin", std::ios::binary);
  PGB_CHECK(f.good(), "sigma.bin not found in the working directory");
  PGB_CHECK(read_record(f, &mu, 8), "sigma.bin: missing mu record");
  PGB_CHECK(read_record(f, &mu_old, 8), "sigma.bin: missing mu_old record");
  // peek the length of the sigma record to report a mesh mismatch clearly
  int32_t n = 0;
  std::streampos pos = f.tellg();
  f.read((char*)&n, 4);
  f.seekg(pos);
  if ((size_t)n != sig.size() * sizeof(double2)) {
    throw Error("io_sigma: sigma.bin was written on a different mesh (record of " + std::to_string(n) +
                " bytes); convert the seed with plibs.regrid_sigma_bin first");
  }
  read_record(f, sig.data(), sig.size() * sizeof(double2));
  require_finite(sig.data(), sig.size(), "the Sigma record of sigma.bin");
  // the (temp, Nw, Norb, Nk) record is optional: a missing or truncated one
  // is skipped, as the reference's read with iostat does (fself.f90:761-766)
  double meta[4];
  int32_t m = 0, m2 = 0;
  if (f.read((char*)&m, 4) && m == 32 && f.read((char*)meta, 32) && f.read((char*)&m2, 4) && m2 == 32) {
    if ((int)std::lround(meta[1]) != Nw || (int)std::lround(meta[2]) != Norb || (int)std::lround(meta[3]) != Nk)
      throw Error("io_sigma: sigma.bin was written on a different mesh; convert the seed with "
                  "plibs.regrid_sigma_bin first");
    if (std::fabs(meta[0] - temp) > 1e-10)
      log("io_sigma: seed was written at T=%10.6f eV, reused raw at T=%10.6f eV (T-annealing)\n", meta[0], temp);
  }
}

// ------------------------------------------------------- host eigen (m x m)
// eigenvalues and the zgeev-normalized eigenvector of eigenvalue idx
void eig_small(const std::vector<double2>& H, int m, std::vector<double2>& w) {
  std::vector<double2> A(H);
  w.assign(m, make_double2(0, 0));
  PGB_CHECK(eigvals_general(A.data(), m, w.data()) >= 0, "Hessenberg eigenvalue iteration did not converge");
}

std::vector<double2> eigvec(const std::vector<double2>& H, int m, double2 lam) {
  std::vector<double2> x(m, make_double2(1.0, 0.0));
  const double sc = 1e-13 * (std::fabs(lam.x) + std::fabs(lam.y) + 1.0);
  for (int it = 0; it < 4; ++it) {
    std::vector<double2> A(m * m), b(x);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) A[i * m + j] = H[i * m + j] - ((i == j) ? (lam + make_double2(sc, 0)) : make_double2(0, 0));
    // complex LU with partial pivoting
    for (int k = 0; k < m; ++k) {
      int p = k;
      for (int i = k + 1; i < m; ++i)
        if (cabs1(A[i * m + k]) > cabs1(A[p * m + k])) p = i;
      if (cabs1(A[p * m + k]) == 0) A[p * m + k] = make_double2(1e-300, 0);
      if (p != k) {
        for (int j = 0; j < m; ++j) std::swap(A[k * m + j], A[p * m + j]);
        std::swap(b[k], b[p]);
      }
      for (int i = k + 1; i < m; ++i) {
        double2 l = cdiv(A[i * m + k], A[k * m + k]);
        for (int j = k; j < m; ++j) A[i * m + j] -= l * A[k * m + j];
        b[i] -= l * b[k];
      }
    }
    for (int k = m - 1; k >= 0; --k) {
      double2 s = b[k];
      for (int j = k + 1; j < m; ++j) s -= A[k * m + j] * b[j];
      b[k] = cdiv(s, A[k * m + k]);
    }
    double nrm = 0;
    for (auto& v : b) nrm += abs2(v);
    nrm = std::sqrt(nrm);
    for (int i = 0; i < m; ++i) x[i] = b[i] * (1.0 / nrm);
  }
  // largest component real and positive (zgeev normalization)
  int kmax = 0;
  for (int i = 1; i < m; ++i)
    if (abs2(x[i]) > abs2(x[kmax])) kmax = i;
  const double a = std::sqrt(abs2(x[kmax]));
  const double2 ph = conj(x[kmax]) * (1.0 / a);
  for (auto& v : x) v = v * ph;
  return x;
}

}  // namespace

const LastStats& last_stats() { return g_stats; }

// ================================================================ inputs ==
void upload_inputs(Inputs& in, const int64_t* kmap, const int64_t* invk, const int64_t* olist, int64_t Nx, int64_t Ny,
                   int64_t Nz, int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Norb, int64_t Nchi, const double* Smat,
                   const double* Cmat, const double2* hamk, const double* eig, const double2* uni) {
  PGB_CHECK(Nkall == Nx * Ny * Nz, "Nkall differs from Nx*Ny*Nz");
  in.Norb = (int)Norb;
  in.Nchi = (int)Nchi;
  in.Nk = (int)Nk;
  in.Nw = (int)Nw;
  build_geom(in.g, kmap, invk, Nx, Ny, Nz, Nk, Nw, Norb, Nchi);
  build_pairs(in.p, olist, (int)Norb, (int)Nchi);
  in.S.alloc(Nchi * Nchi);
  in.C.alloc(Nchi * Nchi);
  in.S.upload(Smat, Nchi * Nchi);
  in.C.upload(Cmat, Nchi * Nchi);
  if (eig) {
    in.eig.alloc(Norb * Nk);
    in.eig.upload(eig, Norb * Nk);
  }
  if (hamk) {
    in.H.alloc(Norb * Norb * Nk);
    in.H.upload(hamk, Norb * Norb * Nk);
  }
  if (uni) {
    in.uni.alloc(Norb * Norb * Nk);
    in.uni.upload(uni, Norb * Norb * Nk);
  }
}

// ================================================================ mkself ==
// One bulk step of the FLEX loop: chi0 (plain or tail-corrected) -> Stoner
// factor (and the sw_rescale clamp) -> V_sigma -> Sigma (FP64 out).  Each of
// the three stages runs in FP32 or FP64 (bit 0 chi0, bit 1 vertex, bit 2
// Sigma set = FP32); chi is converted between the stages where they differ.
template <typename R>
double stage_chi0(Inputs& in, const FlexParams& a, const double2* G, double mu, cx<R>* chi) {
  const Geom& g = in.g;
  Timer tm;
  tm.start();
  TailRef tail{in.eig.p, in.uni.p, mu};
  chi0<R>(g, in.p, G, a.temp, a.sw_tail ? &tail : nullptr, chi);
  g_stats.t_chi0 += tm.stop();
  double sdw = 0, cdw = 0;
  int qs = 0, qc = 0;
  tm.start();
  if (in.soc) {  // max Re eig(-chi0(q,0) V) (fchi0withsoc.f90:156-198)
    stoner<R>(g, chi, in.Vneg.p, in.Vneg.p, &sdw, &cdw, &qs, &qc);
    ckchi_print_soc(g, sdw, qs);
  } else {
    stoner<R>(g, chi, in.S.p, in.C.p, &sdw, &cdw, &qs, &qc);
    ckchi_print(g, sdw, cdw, qs, qc);
  }
  if (a.sw_rescale && sdw >= 1.0) {
    const double rt = 1.0 - 1.0e-4;
    log("[FLEX] Stoner factor=%10.6f >= 1: rescaling chi0 to%7.4f\n", sdw, rt);
    scale_chi<R>(chi, g.K * in.Nchi * in.Nchi, rt / sdw);
  }
  g_stats.t_stoner += tm.stop();
  return sdw;
}
template <typename R>
void stage_vertex(Inputs& in, cx<R>* chi) {
  Timer tm;
  tm.start();
  if (in.soc) {
    PGB_CHECK((std::is_same<R, double>::value), "the spin-orbit loop runs in FP64");
    PGB_CHECK(vertex_soc(reinterpret_cast<double2*>(chi), in.g.K, in.Nchi, in.V.p), "zgesv failed in V_sigma");
  } else {
    PGB_CHECK(vertex<R>(chi, in.g.K, in.g.K, in.Nchi, in.S.p, in.C.p, 0), "zgesv failed in V_sigma");
  }
  g_stats.t_vertex += tm.stop();
}
template <typename R>
void stage_sigma(Inputs& in, const FlexParams& a, const double2* G, const cx<R>* chi, double2* sig) {
  Timer tm;
  tm.start();
  if (in.soc) sigma<R>(in.g, in.p, G, chi, in.Vneg.p, nullptr, a.temp, sig);  // static slot -V
  else sigma<R>(in.g, in.p, G, chi, in.S.p, in.C.p, a.temp, sig);
  g_stats.t_sigma += tm.stop();
}

// the chi buffer of each bulk type, allocated on first use
struct ChiBufs {
  DBuf<float2> f32;
  DBuf<double2> f64;
  DBuf<cdf> fdf;
  void* get(int prec, long long n) {
    if (prec == 32) { if (!f32.p) f32.alloc(n); return f32.p; }
    if (prec == 64) { if (!f64.p) f64.alloc(n); return f64.p; }
    if (!fdf.p) fdf.alloc(n);
    return fdf.p;
  }
  void keep_only(const StagePrec& sp) {
    auto used = [&](int p) { return sp.chi0 == p || sp.vertex == p || sp.sigma == p; };
    if (!used(32)) f32.release();
    if (!used(64)) f64.release();
    if (!used(48)) fdf.release();
  }
};

void convert_chi(void* out, int to, const void* in, int from, long long n) {
  if (to == from) return;
  if (to == 32 && from == 64) convert<float, double>((float2*)out, (const double2*)in, n);
  else if (to == 64 && from == 32) convert<double, float>((double2*)out, (const float2*)in, n);
  else if (to == 32 && from == 48) convert<float, dfl>((float2*)out, (const cdf*)in, n);
  else if (to == 48 && from == 32) convert<dfl, float>((cdf*)out, (const float2*)in, n);
  else if (to == 64 && from == 48) convert<double, dfl>((double2*)out, (const cdf*)in, n);
  else convert<dfl, double>((cdf*)out, (const double2*)in, n);
}

// Bosonic frequencies whose vertex the middle phase of the mixed schedule
// solves in double-float although the rest of its vertex is FP32
// (PYRPA_GB_MID_DF_NU; 0 = none).  Near the magnetic instability the
// matrices I - chi0 S of the lowest frequencies are the ill-conditioned ones,
// and an FP32 solve of them moves the middle phase's fixed point.
int mid_df_nu() {
  const char* s = std::getenv("PYRPA_GB_MID_DF_NU");
  return s ? std::max(0, std::atoi(s)) : kMidDfNu;
}

double flex_bulk(Inputs& in, const FlexParams& a, const double2* G, double mu, const StagePrec& sp, ChiBufs& b,
                 double2* sig) {
  const long long K = in.g.K, KC = K * in.Nchi * in.Nchi;
  PGB_CHECK(sp.vertex == 32 || sp.vertex == 64 || sp.vertex == 48, "the vertex stage runs in FP32, FP64 or double-float");
  void* c0 = b.get(sp.chi0, KC);
  double sdw = 0;
  if (sp.chi0 == 32) sdw = stage_chi0<float>(in, a, G, mu, (float2*)c0);
  else if (sp.chi0 == 64) sdw = stage_chi0<double>(in, a, G, mu, (double2*)c0);
  else sdw = stage_chi0<dfl>(in, a, G, mu, (cdf*)c0);
  // middle phase: the lowest frequencies' vertex in double-float, from the
  // double-float chi0, into a compact buffer [element][matrix]
  const long long nlow = (sp.chi0 == 48 && sp.vertex == 32 && sp.sigma == 48 && !in.soc)
                             ? std::min<long long>((long long)mid_df_nu() * in.Nk, K) : 0;
  DBuf<cdf> low;
  const size_t nel = (size_t)in.Nchi * in.Nchi;
  if (nlow > 0) {
    Timer tl;
    tl.start();
    low.alloc(nlow * (long long)nel);
    PGB_CUDA(cudaMemcpy2DAsync(low.p, nlow * sizeof(cdf), c0, K * sizeof(cdf), nlow * sizeof(cdf), nel,
                               cudaMemcpyDeviceToDevice, ctx().stream));
    PGB_CHECK(vertex<dfl>(low.p, nlow, nlow, in.Nchi, in.S.p, in.C.p, 0), "zgesv failed in V_sigma");
    g_stats.t_vertex += tl.stop();
  }
  void* cv = b.get(sp.vertex, KC);
  convert_chi(cv, sp.vertex, c0, sp.chi0, KC);
  if (sp.vertex == 32) stage_vertex<float>(in, (float2*)cv);
  else if (sp.vertex == 48) stage_vertex<dfl>(in, (cdf*)cv);
  else stage_vertex<double>(in, (double2*)cv);
  void* cs = b.get(sp.sigma, KC);
  convert_chi(cs, sp.sigma, cv, sp.vertex, KC);
  if (nlow > 0)
    PGB_CUDA(cudaMemcpy2DAsync(cs, K * sizeof(cdf), low.p, nlow * sizeof(cdf), nlow * sizeof(cdf), nel,
                               cudaMemcpyDeviceToDevice, ctx().stream));
  if (sp.sigma == 32) stage_sigma<float>(in, a, G, (const float2*)cs, sig);
  else if (sp.sigma == 64) stage_sigma<double>(in, a, G, (const double2*)cs, sig);
  else stage_sigma<dfl>(in, a, G, (const cdf*)cs, sig);
  return sdw;
}

// Stages that the middle phase of the mixed schedule keeps on FP32 bulk:
// PYRPA_GB_FINISH_FP32_STAGES, a comma list of chi0, vertex, sigma or
// "none" (default "vertex").
int mix_finish_mask() {
  const char* s = std::getenv("PYRPA_GB_FINISH_FP32_STAGES");
  if (!s) return 2;
  const std::string v(s);
  return (v.find("chi0") != std::string::npos ? 1 : 0) | (v.find("vertex") != std::string::npos ? 2 : 0) |
         (v.find("sigma") != std::string::npos ? 4 : 0);
}

// Bulk type of the middle phase's other stages: double-float (default) or,
// with PYRPA_GB_FINISH_BULK=fp64, FP64.
int mix_finish_bulk() {
  const char* s = std::getenv("PYRPA_GB_FINISH_BULK");
  return (s && std::string(s) == "fp64") ? 64 : 48;
}

// Stage types of the judging phase of the mixed schedule
// (PYRPA_GB_JUDGE_BULK): "df" (default) double-float chi0, vertex and Sigma,
// about 1e-13 relative; "df64" the same with the FP64 vertex; "fp64" FP64
// throughout.
StagePrec mix_judge_prec() {
  const char* s = std::getenv("PYRPA_GB_JUDGE_BULK");
  const std::string v = s ? s : "df";
  if (v == "fp64") return StagePrec{64, 64, 64};
  if (v == "df64") return StagePrec{48, 64, 48};
  return StagePrec{48, 48, 48};
}

// PYRPA_GB_MIX_DIIS=keep keeps the FP32-phase DIIS history across the switch
// to the middle phase's wider bulk (default: a fresh history)
bool mix_diis_reset() {
  const char* s = std::getenv("PYRPA_GB_MIX_DIIS");
  return !(s && std::string(s) == "keep");
}

// The judging phase of the mixed schedule.  The middle phase's iterates come
// from an FP32 vertex (double-float for its lowest frequencies, mid_df_nu),
// whose fixed point differs from the FP64 one: on c2 by 1.7e-6 of max|Sigma|,
// mostly at high Matsubara frequencies.  The judging phase keeps the middle
// phase's DIIS history (PYRPA_GB_JUDGE_DIIS=fresh starts a new one, which
// removes the bias through about five more judging iterations).
// PYRPA_GB_JUDGE_POLISH takes that many full steps of the judging map without
// DIIS after convergence; on c2 one step cut the Sigma bias to 1.6e-7 but
// moved lambda from 8.8e-8 to 4.7e-7 of the FP64 value, and a second made both
// worse (undamped steps are not contractive near the instability), so the
// default is none.
// PYRPA_GB_JUDGE_MIN is the least number of judging iterations,
// PYRPA_GB_JUDGE_EPS_FACTOR scales eps for the judging test (<= 1).
struct JudgeRule {
  bool fresh = false;
  int min_iterations = 1;
  double eps_factor = 1.0;
  int polish = kJudgePolish;
};
JudgeRule judge_rule() {
  JudgeRule r;
  if (const char* s = std::getenv("PYRPA_GB_JUDGE_DIIS")) r.fresh = std::string(s) == "fresh";
  if (const char* s = std::getenv("PYRPA_GB_JUDGE_POLISH")) r.polish = std::max(0, std::atoi(s));
  if (const char* s = std::getenv("PYRPA_GB_JUDGE_MIN")) r.min_iterations = std::max(1, std::atoi(s));
  if (const char* s = std::getenv("PYRPA_GB_JUDGE_EPS_FACTOR")) r.eps_factor = std::min(1.0, std::atof(s));
  return r;
}

// Stages that the FP32 phase of the FLEX loop runs in FP32 (default all):
// PYRPA_GB_FP32_STAGES is a comma list of chi0, vertex, sigma.
int fp32_stage_mask() {
  const char* s = std::getenv("PYRPA_GB_FP32_STAGES");
  if (!s) return 7;
  const std::string v(s);
  return (v.find("chi0") != std::string::npos ? 1 : 0) | (v.find("vertex") != std::string::npos ? 2 : 0) |
         (v.find("sigma") != std::string::npos ? 4 : 0);
}

// prec: 64 FP64 bulk, 48 double-float chi0 and Sigma, 32 FP32 bulk,
// kPrecMixed the three-phase schedule: FP32 bulk until the residual reaches
// the FP32 rounding floor, then double-float chi0 and Sigma with an FP32
// vertex, then the judging iterations (double-float throughout by default,
// mix_judge_prec); convergence is only declared in the judging phase.
void mkself_core(Inputs& in, const FlexParams& a, double2* sig_out, double* mu_out, const double2* seed,
                 double seed_mu, double seed_mu_old, int prec) {
  cudaStream_t st = ctx().stream;
  const Geom& g = in.g;
  const Pairs& p = in.p;
  const int Norb = in.Norb, Nchi = in.Nchi, Nk = in.Nk, Nw = in.Nw;
  PGB_CHECK(a.m_diis >= 1 && a.m_diis <= 16, "m_diis outside 1..16");
  const long long K = g.K, No2 = (long long)Norb * Norb, KE = K * No2;
  DBuf<double>& S = in.S;
  DBuf<double>& C = in.C;
  DBuf<double>& eig = in.eig;
  DBuf<double2>& H = in.H;
  DBuf<double2>& uni = in.uni;
  DBuf<double2> G(KE), sig(KE), sig0(KE), eg((size_t)K * Norb);
  const int mask32 = fp32_stage_mask();
  std::vector<DBuf<double2>> xout(a.m_diis), res(a.m_diis);
  for (int i = 0; i < a.m_diis; ++i) {
    xout[i].alloc(KE);
    res[i].alloc(KE);
  }
  double mu = a.mu_init, mu_old = 0.0, esterr = 0.0, maxchi0s = 0.0;
  if (a.sw_in || seed) {
    if (seed) {
      mu = seed_mu;
      mu_old = seed_mu_old;
      PGB_CUDA(cudaMemcpyAsync(sig.p, seed, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    } else {
      log(" load self\n");
      std::vector<double2> hs(KE);
      read_sigma_bin(mu, mu_old, hs, a.temp, Nw, Norb, Nk);
      sig.upload(hs.data(), KE);
    }
    if (a.sigma_scale != 1.0) {
      log("[FLEX] scale loaded sigma seed by%10.6f\n", a.sigma_scale);
      scal(sig.p, a.sigma_scale, KE);
    }
    PGB_CUDA(cudaMemcpyAsync(sig0.p, sig.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    PGB_CHECK(dyson(G.p, sig.p, H.p, mu, a.temp, Nk, Nw, Norb), "singular G^-1 in the Dyson step");
  } else {
    mu_old = mu * 1.2;
    sig0.zero();
    green0(G.p, eig.p, uni.p, mu, a.temp, Nk, Nw, Norb);
  }
  // DIIS state
  int n_hist = 0, i_hist = 0;
  std::vector<double> Bc((size_t)a.m_diis * a.m_diis, 0.0);
  // mu bracket cache
  bool bracket_valid = false;
  double muS_cache = 0, muL_cache = 0;
  DBuf<double> partmax(1024), dmax(1);

  auto compare_sigma = [&]() {
    i_hist = i_hist % a.m_diis + 1;
    n_hist = std::min(n_hist + 1, (int)a.m_diis);
    const int slot = i_hist - 1;
    PGB_CUDA(cudaMemcpyAsync(xout[slot].p, sig.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    k_sub<<<nblocks(KE, 256) > 65536 ? 65536 : nblocks(KE, 256), 256, 0, st>>>(res[slot].p, sig.p, sig0.p, KE);
    launch_check("diis_residual");
    ctx().kernel_launches++;
    const int n = n_hist;
    std::vector<int> idx(n);
    for (int h = 1; h <= n; ++h) idx[h - 1] = (((i_hist - n + h - 1) % a.m_diis) + a.m_diis) % a.m_diis;
    for (int h = 0; h < n; ++h) {
      const double v = dot_re(res[slot].p, res[idx[h]].p, KE);
      Bc[slot * a.m_diis + idx[h]] = v;
      Bc[idx[h] * a.m_diis + slot] = v;
    }
    const int nn = n + 1;
    std::vector<double> B((size_t)nn * nn, 0.0), c(nn, 0.0);
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) B[i * nn + j] = Bc[idx[i] * a.m_diis + idx[j]];
      B[i * nn + n] = 1.0;
      B[n * nn + i] = 1.0;
      B[i * nn + i] += 1.0e-12;
    }
    c[n] = 1.0;
    if (!solve_real(B, c, nn)) {
      log(" DIIS: dgesv failed, fallback to most-recent entry\n");
      std::fill(c.begin(), c.end(), 0.0);
      c[n - 1] = 1.0;
    }
    DiisTerms t{};
    for (int h = 0; h < n; ++h) {
      t.x[h] = xout[idx[h]].p;
      t.c[h] = c[h];
    }
    k_diis_mix<<<1024, 256, 0, st>>>(sig.p, sig0.p, t, n, a.pp, n >= 2 ? 1 : 0, partmax.p, KE);
    launch_check("diis_mix");
    k_max_parts<<<1, 256, 0, st>>>(dmax.p, partmax.p, 1024);
    launch_check("max_parts");
    ctx().kernel_launches += 2;
    dmax.download(&esterr, 1);
    sync();
    log("esterr=%9.2E\n", esterr);
  };

  auto get_rn = [&](double rmu) { return filling_cp(eg.p, eig.p, Nk, Nw, Norb, rmu, a.temp); };

  auto renew_mu = [&]() {
    charpoly_gk(eg.p, H.p, sig.p, Nk, Nw, Norb);
    const double eps = (esterr > 1.0e-2) ? 1.0e-8 : esterr * 1.0e-1;
    double dmu = std::fabs(mu - mu_old) * 2.0;
    if (dmu < eps * 4.0) dmu = eps * 4.0;
    mu_old = mu;
    const double fill = a.fill;
    double muS = 0, muL = 0, rnS = 0, rnL = 0;
    bool found = false;
    if (bracket_valid) {
      rnS = get_rn(muS_cache);
      rnL = get_rn(muL_cache);
      if (rnS < fill && rnL > fill) {
        muS = muS_cache;
        muL = muL_cache;
        found = true;
        log("[mu] cached bracket valid\n");
      } else {
        log("[mu] cached bracket invalid, re-searching\n");
      }
    }
    if (!found) {
      muL = mu + dmu;
      muS = mu - dmu;
      for (int it = 1; it <= 100; ++it) {
        mu = muL;
        rnL = get_rn(mu);
        if (rnL < fill) {
          if (std::fabs(fill - rnL) > 0.5) muL += 1.0;
          else if (std::fabs(fill - rnL) > dmu) muL += 0.5;
          else muL += dmu;
        } else {
          break;
        }
        PGB_CHECK(it < 100, "Too many");
      }
      for (int it = 1; it <= 100; ++it) {
        mu = muS;
        rnS = get_rn(mu);
        if (rnS > fill) {
          if (std::fabs(rnS - fill) > 0.5) muS -= 1.0;
          else if (std::fabs(rnS - fill) > dmu) muS -= 0.5;
          else muS -= dmu;
        } else {
          break;
        }
        PGB_CHECK(it < 100, "Too many");
      }
    }
    muS_cache = muS;
    muL_cache = muL;
    bracket_valid = true;
    rnL -= fill;
    rnS -= fill;
    double rnc = rnS, muc = muS, mud = 0.0, muM = 0.0, rnM = 0.0;
    bool flag = false;
    // inverse quadratic interpolation / bisection hybrid (fself.f90:623-654)
    for (int it = 1; it <= 100; ++it) {
      if (rnc != rnS && rnc != rnL)
        muM = (muL * rnS * rnc * (rnS - rnc) + muS * rnL * rnc * (rnc - rnL) + muc * rnL * rnS * (rnL - rnS)) /
              ((rnL - rnS) * (rnc - rnL) * (rnc - rnS));
      else
        muM = muL - rnL * (muL - muS) / (rnL - rnS);
      if ((0.25 * (3.0 * muS + muL) > muM || muM > muL) || (flag && std::fabs(muM - muL) >= std::fabs(muL - muc) * 0.5) ||
          (!flag && std::fabs(muM - muL) >= std::fabs(muc - mud) * 0.5) || (flag && std::fabs(muL - muc) < 1.0e-8) ||
          (!flag && std::fabs(muc - mud) < 1.0e-8)) {
        muM = (muL + muS) * 0.5;
        flag = true;
      } else {
        flag = false;
      }
      if (std::fabs(muL - muM) < eps) break;
      mu = muM;
      rnM = get_rn(muM);
      mud = muc;
      muc = muL;
      rnc = rnL;
      if (rnS * (rnM - fill) < 0) {
        muL = muM;
        rnL = rnM - fill;
      } else {
        muS = muM;
        rnS = rnM - fill;
      }
      if (std::fabs(rnS) < std::fabs(rnL)) {
        std::swap(muL, muS);
        std::swap(rnL, rnS);
      }
      PGB_CHECK(it < 100, "Too many loop!");
    }
    mu = (rnL == rnS) ? (muS + muL) * 0.5 : (muS * rnL - muL * rnS) / (rnL - rnS);
    rnM = get_rn(mu);
    mu_old = mu;
    log("mu  =%8.4f filling =%8.4f\n", mu, rnM);
  };

  Timer tm;
  int it = 0;
  // Mixed schedule, three phases:
  //   0  the stages in mask32 on FP32 bulk (default all);
  //   1  chi0 and Sigma on FP64 bulk, the stages in finish_mask (default the
  //      vertex) still on FP32: the FP32 rounding floor of the residual comes
  //      from the chi0 and Sigma convolutions, not from the vertex solve;
  //   2  the judging phase: FP64, or in the mixed mode the stage types of
  //      mix_judge_prec (default double-float throughout).
  // A phase ends when the residual is below eps, below kMixSwitch (phase 0
  // only) or, once it is below kMixStallFrom, has not reached a new minimum
  // for kMixStall iterations.  Convergence is declared only in phase 2.
  const int finish_mask = mix_finish_mask();
  const int finish_bulk = mix_finish_bulk();
  int phase = (prec == kPrecMixed || prec == 32) ? 0 : 2;
  const StagePrec judge = prec == kPrecMixed ? mix_judge_prec() : StagePrec{64, 64, 64};
  auto prec_of = [&](int ph) {
    if (prec == kPrecDF) return StagePrec{48, 64, 48};
    auto pick = [&](int bit, int other) { return (ph == 0 ? mask32 : finish_mask) & bit ? 32 : other; };
    if (ph == 2) return judge;
    const int other = ph == 0 ? 64 : finish_bulk;
    return StagePrec{pick(1, other), pick(2, 64), pick(4, other)};
  };
  ChiBufs bufs;
  double best = 1e300;
  int since_best = 0;
  const JudgeRule judge_r = judge_rule();
  int judged = 0;  // iterations of the mixed schedule's judging phase
  for (it = 1; it <= a.scf_loop; ++it) {
    log("iter=%5d\n", it);
    maxchi0s = flex_bulk(in, a, G.p, mu, prec_of(phase), bufs, sig.p);
    tm.start();
    if (a.sub_sigma > 0) hf_subtract(sig.p, Nk, Nw, Norb, (int)a.sub_sigma);
    compare_sigma();
    g_stats.t_diis += tm.stop();
    g_stats.esterr = esterr;
    g_stats.iterations = it;
    g_stats.stoner = maxchi0s;
    if (phase == 0) g_stats.iterations32 = it;
    if (phase == 1) ++g_stats.iterations_finish32;
    if (prec != kPrecMixed) {
      if (esterr < a.eps) break;
    } else if (phase == 2) {
      ++judged;
      if (esterr < a.eps * judge_r.eps_factor && judged >= judge_r.min_iterations) break;
    } else {
      // the stall count starts once the residual is out of the initial transient
      if (esterr < best * 0.9) {
        best = esterr;
        since_best = 0;
      } else if (best < kMixStallFrom) {
        ++since_best;
      }
      const bool next = esterr < a.eps || (phase == 0 && esterr < kMixSwitch) || since_best >= kMixStall;
      if (next && phase == 0 && a.stop_at_fp32_floor) break;
      if (next) {
        const int from = phase;
        phase = (phase == 0 && finish_mask != 0) ? 1 : 2;
        log("[FLEX] residual%9.2E: continuing with %s\n", esterr,
            phase == 1 ? "wider chi0 and Sigma, FP32 vertex" : "the judging iterations");
        if ((from == 0 && mix_diis_reset()) || (phase == 2 && judge_r.fresh)) {
          // the FP32 entries carry the FP32 rounding floor in their residuals,
          // the middle phase's the FP32 vertex's fixed point: the later phases
          // start a fresh history from the current Sigma
          n_hist = 0;
          i_hist = 0;
        }
        best = 1e300;
        since_best = 0;
        bufs.keep_only(prec_of(phase));
      }
    }
    tm.start();
    renew_mu();
    g_stats.t_mu += tm.stop();
    tm.start();
    PGB_CHECK(dyson(G.p, sig.p, H.p, mu, a.temp, Nk, Nw, Norb), "singular G^-1 in the Dyson step");
    PGB_CUDA(cudaMemcpyAsync(sig0.p, sig.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    g_stats.t_dyson += tm.stop();
  }
  if (prec == kPrecMixed && phase == 2 && esterr < a.eps) {
    // full steps of the judging map from the converged Sigma, without DIIS
    for (int k = 0; k < judge_r.polish; ++k) {
      tm.start();
      renew_mu();
      g_stats.t_mu += tm.stop();
      tm.start();
      PGB_CHECK(dyson(G.p, sig.p, H.p, mu, a.temp, Nk, Nw, Norb), "singular G^-1 in the Dyson step");
      g_stats.t_dyson += tm.stop();
      maxchi0s = flex_bulk(in, a, G.p, mu, prec_of(2), bufs, sig.p);
      if (a.sub_sigma > 0) hf_subtract(sig.p, Nk, Nw, Norb, (int)a.sub_sigma);
      g_stats.stoner = maxchi0s;
      ++g_stats.judge_polish;
    }
  }
  if (maxchi0s >= 1.0) {
    log("[FLEX] WARNING: Stoner factor >= 1 at the final iteration:\n");
    log("[FLEX]   max eig[chi0*S] =%10.6f -> the normal state is magnetically unstable at this T/U.\n", maxchi0s);
  }
  std::vector<double2> hs(KE);
  if (a.sw_out) {
    sig.download(hs.data(), KE);
    sync();
    write_sigma_bin(mu, mu_old, hs, a.temp, Nw, Norb, Nk);
  }
  tm.start();
  renew_mu();
  g_stats.t_mu += tm.stop();
  PGB_CUDA(cudaMemcpyAsync(sig_out, sig.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  sync();
  *mu_out = mu;
  g_stats.mu = mu;
}

void run_mkself(const MkselfArgs& a, int prec) {
  g_stats = LastStats{};
  Inputs in;
  upload_inputs(in, a.kmap, a.invk, a.olist, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Smat, a.Cmat,
                a.hamk, a.eig, a.uni);
  FlexParams prm{a.mu_init, a.fill, a.temp, a.scf_loop, a.pp, a.eps, a.sub_sigma, a.sw_out, a.sw_in, a.m_diis,
                 a.sw_rescale, a.sw_tail, a.sigma_scale};
  const long long KE = in.g.K * a.Norb * a.Norb;
  DBuf<double2> sig(KE);
  mkself_core(in, prm, sig.p, a.mu_out, nullptr, 0.0, 0.0, prec);
  sig.download(a.sigmak, KE);
  sync();
}

// Two-pass Arnoldi of lin_eliash (feliash.f90:190-388, feliashwithsoc.f90:190-388):
// pass 1 from the initial gap, exit at a Ritz value >= 0.1, else pass 2 with
// the shift -lambda_- and that Ritz vector deflated.  apply_op/inner/norm/init
// define the operator and the inner product of the caller's vector space of n
// elements; the normalized Ritz vector goes to delta_out, lambda is returned.
// With a restart tolerance set, refine(residual / |lambda|) is asked after
// every cycle whether the operator has just been replaced by a more precise
// one (true: the pass restarts on it from the current Ritz vector, whatever
// the residual).
template <class Apply, class Inner, class Norm, class Init, class Refine>
double arnoldi_two_pass(int m, long long KE, Apply apply_op, Inner inner, Norm norm, Init init_vec,
                        double2* delta_out, Refine refine) {
  cudaStream_t st = ctx().stream;
  double lambda_out = 0.0;
  DBuf<double2> w(KE);
  PGB_CHECK(m <= 64, "arnoldi_m above 64 is not supported");
  std::vector<DBuf<double2>> V(m);
  for (auto& v : V) v.alloc(KE);
  DBuf<double2> D(KE);
  auto arnoldi = [&](double shift, const double2* defl, std::vector<double2>& Hm, int& m_act) {
    Hm.assign((size_t)(m + 1) * m, make_double2(0, 0));
    m_act = m;
    for (int j = 0; j < m; ++j) {
      apply_op(w.p, V[j].p);
      if (defl) {
        axpy(w.p, make_double2(shift, 0), V[j].p, KE);
        double2 h = inner(defl, w.p);
        axpy(w.p, make_double2(-h.x, -h.y), defl, KE);
      }
      for (int ii = 0; ii <= j; ++ii) {
        double2 h = inner(V[ii].p, w.p);
        Hm[ii * m + j] = h;
        axpy(w.p, make_double2(-h.x, -h.y), V[ii].p, KE);
      }
      const double beta = norm(w.p);
      Hm[(j + 1) * m + j] = make_double2(beta, 0);
      if (beta < 1.0e-14) {
        m_act = j + 1;
        break;
      }
      if (j < m - 1) {
        PGB_CUDA(cudaMemcpyAsync(V[j + 1].p, w.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(V[j + 1].p, 1.0 / beta, KE);
      }
    }
  };
  // Ritz vector of lam into out (unit norm); returns the Ritz residual
  // |h_{m+1,m}| |y_m| / |y| of the pair
  auto ritz = [&](double2* out, const std::vector<double2>& Hm, int m_act, double2 lam) {
    std::vector<double2> Hs((size_t)m_act * m_act);
    for (int i = 0; i < m_act; ++i)
      for (int j = 0; j < m_act; ++j) Hs[i * m_act + j] = Hm[i * m + j];
    std::vector<double2> y = eigvec(Hs, m_act, lam);
    std::vector<const double2*> xs(m_act);
    for (int i = 0; i < m_act; ++i) xs[i] = V[i].p;
    lincomb(out, xs.data(), y.data(), m_act, KE);
    scal(out, 1.0 / norm(out), KE);
    double yn = 0;
    for (const auto& v : y) yn += abs2(v);
    return Hm[(size_t)m_act * m + m_act - 1].x * std::sqrt(abs2(y[m_act - 1]) / std::max(yn, 1e-300));
  };
  auto ritz_values = [&](const std::vector<double2>& Hm, int m_act) {
    std::vector<double2> Hs((size_t)m_act * m_act), ev;
    for (int i = 0; i < m_act; ++i)
      for (int j = 0; j < m_act; ++j) Hs[i * m_act + j] = Hm[i * m + j];
    eig_small(Hs, m_act, ev);
    return ev;
  };
  // with a tolerance set, restart a pass from its Ritz vector (in D) until the
  // residual over |lambda| is below it; returns lambda on the operator's scale
  const double tol = ctx().arnoldi_tol;
  constexpr int kMaxCycles = 12;
  auto converge = [&](double shift, const double2* defl, std::vector<double2>& Hm, int& m_act,
                      std::vector<double2>& ev, int& imax, double res) {
    int cycles = 1;
    double lam = ev[imax].x - shift;
    while (tol > 0.0 && cycles < kMaxCycles) {
      const bool switched = refine(res / std::max(std::fabs(lam), 1e-300));
      if (!switched && res <= tol * std::fabs(lam)) break;
      PGB_CUDA(cudaMemcpyAsync(V[0].p, D.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      arnoldi(shift, defl, Hm, m_act);
      ev = ritz_values(Hm, m_act);
      imax = 0;
      for (int i = 1; i < m_act; ++i)
        if (ev[i].x > ev[imax].x) imax = i;
      lam = ev[imax].x - shift;
      res = ritz(D.p, Hm, m_act, ev[imax]);
      ++cycles;
      log("  restart %2d: lambda =%14.10f, residual %9.2e\n", cycles, lam, res / std::max(std::fabs(lam), 1e-300));
    }
    g_stats.ritz_residual = res / std::max(std::fabs(lam), 1e-300);
    g_stats.arnoldi_cycles = cycles;
    return lam;
  };
  // pass 1: no shift
  init_vec(V[0].p);
  log("Arnoldi pass 1 (no shift): Krylov dim =%4d ...\n", m);
  std::vector<double2> Hm;
  int m_act = m;
  arnoldi(0.0, nullptr, Hm, m_act);
  std::vector<double2> ev = ritz_values(Hm, m_act);
  int imin = 0, imax = 0;
  for (int i = 1; i < m_act; ++i) {
    if (ev[i].x < ev[imin].x) imin = i;
    if (ev[i].x > ev[imax].x) imax = i;
  }
  const double lambda1 = ev[imin].x;
  for (int i = 0; i < m_act; ++i) log("%4d%14.6f\n", i + 1, ev[i].x);
  log("  lambda_- =%12.6f\n", lambda1);
  auto keep_ritz = [&](const std::vector<double2>& e, double shift) {
    std::vector<double> r;
    for (const auto& z : e) r.push_back(z.x - shift);
    std::sort(r.begin(), r.end(), [](double x, double y) { return x > y; });
    g_stats.nritz = (int)std::min<size_t>(r.size(), 16);
    for (int i = 0; i < g_stats.nritz; ++i) g_stats.ritz[i] = r[i];
  };
  keep_ritz(ev, 0.0);
  if (ev[imax].x >= 0.1) {
    const double res = ritz(D.p, Hm, m_act, ev[imax]);
    lambda_out = converge(0.0, nullptr, Hm, m_act, ev, imax, res);
    if (g_stats.arnoldi_cycles > 1) keep_ritz(ev, 0.0);
    log("  eliash   =%12.6f\n", lambda_out);
  } else {
    refine(0.0);  // pass 2 runs on the final operator from its first step
    DBuf<double2> delta1(KE);
    ritz(delta1.p, Hm, m_act, ev[imin]);
    const double shift = -lambda1;
    init_vec(V[0].p);
    double2 h = inner(delta1.p, V[0].p);
    axpy(V[0].p, make_double2(-h.x, -h.y), delta1.p, KE);
    const double b0 = norm(V[0].p);
    if (!(b0 >= 1.0e-14)) {
      // the operator has no component outside the pass-1 direction
      lambda_out = lambda1;
      g_stats.ritz_residual = 0.0;
      g_stats.arnoldi_cycles = 1;
      PGB_CUDA(cudaMemcpyAsync(D.p, delta1.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    } else {
      scal(V[0].p, 1.0 / b0, KE);
      log("Arnoldi pass 2 (shift=%10.6f): Krylov dim =%4d ...\n", shift, m);
      arnoldi(shift, delta1.p, Hm, m_act);
      ev = ritz_values(Hm, m_act);
      imax = 0;
      for (int i = 1; i < m_act; ++i)
        if (ev[i].x > ev[imax].x) imax = i;
      for (int i = 0; i < m_act; ++i) log("%4d%14.6f\n", i + 1, ev[i].x - shift);
      const double res = ritz(D.p, Hm, m_act, ev[imax]);
      lambda_out = converge(shift, delta1.p, Hm, m_act, ev, imax, res);
      keep_ritz(ev, shift);
      log("  eliash   =%12.6f\n", lambda_out);
    }
  }
  PGB_CUDA(cudaMemcpyAsync(delta_out, D.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  sync();
  return lambda_out;
}

template <class Apply, class Inner, class Norm, class Init>
double arnoldi_two_pass(int m, long long KE, Apply apply_op, Inner inner, Norm norm, Init init_vec,
                        double2* delta_out) {
  return arnoldi_two_pass(m, KE, apply_op, inner, norm, init_vec, delta_out, [](double) { return false; });
}

// FP32 start of the double-float Eliashberg stage of the mixed schedule:
// PYRPA_GB_ELIASH_FP32=n runs at most n FP32 cycles (off by default: on c2
// an FP32 application costs about half a double-float one, and two FP32
// cycles plus one double-float cycle took longer than two double-float ones)
int eliash_fp32_cycles() {
  const char* e = std::getenv("PYRPA_GB_ELIASH_FP32");
  return e ? std::max(0, std::atoi(e)) : kEliashFp32Cycles;
}

// V_Delta in the bulk type of the Eliashberg stage; for double-float the
// solve runs in double-float, or in FP64 with PYRPA_GB_ELIASH=df64
template <typename R>
bool vertex_delta(cx<R>* chi, long long K, int Nchi, const double* S, const double* C, int mode) {
  const char* e = std::getenv("PYRPA_GB_ELIASH");
  if constexpr (std::is_same<R, dfl>::value) {
    if (!(e && std::string(e) == "df64")) return vertex<dfl>(chi, K, K, Nchi, S, C, mode);
    const long long n = K * Nchi * Nchi;
    DBuf<double2> t(n);
    widen<dfl>(t.p, chi, n);
    const bool ok = vertex<double>(t.p, K, K, Nchi, S, C, mode);
    narrow<dfl>(chi, t.p, n);
    return ok;
  } else {
    return vertex<R>(chi, K, K, Nchi, S, C, mode);
  }
}

// ============================================================ lin_eliash ==
// chi (device, cx<R>) is overwritten with the pairing vertex V_Delta; if
// chi_host is given, V_Delta is also copied back there (feliash.f90:61).
template <typename R>
double eliash_core(Inputs& in, cx<R>* chi, const double2* G, const double* init, const double* prt,
                   const EliashParams& a, double2* delta_out, double2* chi_host) {
  cudaStream_t st = ctx().stream;
  const Geom& g = in.g;
  const Pairs& p = in.p;
  const int Norb = in.Norb, Nchi = in.Nchi, Nk = in.Nk, Nw = in.Nw;
  const long long K = g.K, KE = K * Norb * Norb, KC = K * Nchi * Nchi;
  const bool singlet = a.gap_sym >= 0;
  log(singlet ? "singlet\n" : "triplet\n");
  DBuf<double>& S = in.S;
  DBuf<double>& C = in.C;
  DBuf<double2>& uni = in.uni;
  {
    Timer tv;
    tv.start();
    PGB_CHECK(vertex_delta<R>(chi, K, Nchi, S.p, C.p, singlet ? 1 : 2), "zgesv failed in V_delta");
    g_stats.t_vertex += tv.stop();
    if (chi_host) {
      DBuf<double2> tmp(KC);
      if (std::is_same<R, double>::value)
        PGB_CUDA(cudaMemcpyAsync(tmp.p, chi, KC * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      else widen<R>(tmp.p, chi, KC);
      tmp.download(chi_host, KC);
      sync();
    }
  }
  const double weight = a.temp / (double)g.Nkall;
  const double scale = weight / (double)g.P;
  DeltaKernelCache<R> cache;
  DBuf<double2> F(KE);
  Timer ta;
  // Mixed schedule with a restarted Arnoldi: the first cycles (at most
  // kEliashFp32Cycles, until the Ritz residual is below kEliashFp32Tol of
  // lambda) apply an FP32 copy of the double-float operator, which costs a
  // fraction of a double-float application; the pass then restarts from
  // their Ritz vector on the double-float operator and converges there, so
  // lambda and the gap come from double-float cycles only.  The FP32 V_Delta
  // and its transforms are freed before the double-float transforms are made.
  std::unique_ptr<DBuf<cx<float>>> chi32;
  std::unique_ptr<DeltaKernelCache<float>> cache32;
  int fp32_cycles = 0;
  const int fp32_cap = eliash_fp32_cycles();
  if constexpr (std::is_same<R, dfl>::value) {
    if (ctx().precision == kPrecMixed && ctx().arnoldi_tol > 0.0 && a.arnoldi_m > 0 && fp32_cap > 0) {
      chi32 = std::make_unique<DBuf<cx<float>>>((size_t)KC);
      convert<float, dfl>(chi32->p, chi, KC);
      cache32 = std::make_unique<DeltaKernelCache<float>>();
    }
  }
  // Double-float stage: F = -G Delta G^H in double-float too, from a
  // double-float copy of G (PYRPA_GB_MKFK_DF=0 keeps the FP64 product)
  std::unique_ptr<DBuf<cdf>> Gdf, Fdf;
  if constexpr (std::is_same<R, dfl>::value) {
    const char* e = std::getenv("PYRPA_GB_MKFK_DF");
    std::vector<double> hprt(Norb);
    PGB_CUDA(cudaMemcpyAsync(hprt.data(), prt, sizeof(double) * Norb, cudaMemcpyDeviceToHost, st));
    sync();
    bool signs = true;
    for (double x : hprt) signs = signs && (x == 1.0 || x == -1.0);
    if (!(e && std::string(e) == "0") && signs && Norb <= 5) {
      Gdf = std::make_unique<DBuf<cdf>>((size_t)KE);
      Fdf = std::make_unique<DBuf<cdf>>((size_t)KE);
      convert<dfl, double>(Gdf->p, G, KE);
    }
  }
  auto apply_op = [&](double2* out, const double2* v) {
    ta.start();
    if (chi32) {
      mkfk(F.p, G, v, K, Norb);
      mkdelta<float>(g, p, F.p, chi32->p, S.p, C.p, prt, singlet, scale, out, cache32.get());
    } else if (Fdf) {
      if constexpr (std::is_same<R, dfl>::value) {
        PGB_CHECK(mkfk_df(Fdf->p, Gdf->p, v, K, Norb), "no double-float mkfk for this orbital count");
        mkdelta<R>(g, p, nullptr, chi, S.p, C.p, prt, singlet, scale, out, &cache, Fdf->p);
      }
    } else {
      mkfk(F.p, G, v, K, Norb);
      mkdelta<R>(g, p, F.p, chi, S.p, C.p, prt, singlet, scale, out, &cache);
    }
    g_stats.t_apply += ta.stop();
    g_stats.applies += 1;
  };
  auto refine = [&](double rel) {
    if (!chi32) return false;
    ++fp32_cycles;
    if (rel > kEliashFp32Tol && fp32_cycles < fp32_cap) return false;
    log("  FP32 Arnoldi cycles: %d (residual %9.2e), continuing in double-float\n", fp32_cycles, rel);
    cache32.reset();
    chi32.reset();
    return true;
  };
  auto inner = [&](const double2* u, const double2* v) {
    double2 s = inner_w(u, v, g.kweight.p, Nk, KE);
    return make_double2(2.0 * s.x, 2.0 * s.y);
  };
  auto norm = [&](const double2* f) { return std::sqrt(2.0 * inner_w(f, f, g.kweight.p, Nk, KE).x); };
  auto init_vec = [&](double2* d) {
    initial_delta(d, init, uni.p, Nk, Nw, Norb, (int)a.gap_sym);
    const double nrm = inner_w(d, d, g.kweight.p, Nk, KE).x;
    PGB_CHECK(nrm > 0, "Error: get_initial_delta norm <= 0");
    scal(d, 1.0 / std::sqrt(2.0 * nrm), KE);
  };
  double lambda_out = 0.0;
  const int m = (int)a.arnoldi_m;
  if (m > 0) {
    lambda_out = arnoldi_two_pass(m, KE, apply_op, inner, norm, init_vec, delta_out, refine);
    PGB_CHECK(!chi32, "the FP32 Arnoldi cycles did not hand over to double-float");
  } else {
    // shifted power method with deflation (feliash.f90:66-140)
    DBuf<double2> D(KE), nd(KE), d1(KE), tmp(KE);
    double lambda1 = 0.0, lam_phys = 0.0, lam_rq = 0.0, inrm = 1.0;
    for (int i_eig = 1; i_eig <= 2; ++i_eig) {
      init_vec(D.p);
      if (i_eig == 2) {
        const double proj = inner(d1.p, D.p).x;
        axpy(D.p, make_double2(-proj, 0), d1.p, KE);
        scal(D.p, 1.0 / norm(D.p), KE);
      }
      double lam_prev = 0.0;
      for (int it = 1; it <= a.itemax; ++it) {
        apply_op(nd.p, D.p);
        if (i_eig == 2) {
          axpy(nd.p, make_double2(-lambda1, 0), D.p, KE);
          const double proj = inner(d1.p, nd.p).x;
          axpy(nd.p, make_double2(-proj, 0), d1.p, KE);
        }
        const double nrm = norm(nd.p);
        PGB_CHECK(nrm > 0, "Error: norm <= 0 in iter_loop");
        inrm = 1.0 / nrm;
        lam_rq = inner(D.p, nd.p).x;
        lam_phys = lam_rq + lambda1;
        // vector error: min(||nd/|nd| - D||, ||nd/|nd| + D||)
        PGB_CUDA(cudaMemcpyAsync(tmp.p, nd.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(tmp.p, inrm, KE);
        axpy(tmp.p, make_double2(-1, 0), D.p, KE);
        const double ep = norm(tmp.p);
        axpy(tmp.p, make_double2(2, 0), D.p, KE);
        const double en = norm(tmp.p);
        const double verr = std::min(ep, en);
        log("%4d lambda_elsh=%16.8E%16.8E  vec_err=%12.4E\n", it, lam_phys, std::fabs(lam_phys - lam_prev), verr);
        if (lam_phys < 0.0 && verr < a.eps) break;
        if (verr < a.eps && std::fabs(lam_phys - lam_prev) < a.eps * (std::fabs(lam_phys) + 1e-10)) break;
        lam_prev = lam_phys;
        PGB_CUDA(cudaMemcpyAsync(D.p, nd.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(D.p, inrm, KE);
      }
      if (i_eig == 1) {
        if (lam_phys > 0.0) {
          lambda_out = lam_phys;
          break;
        }
        lambda1 = lam_rq;
        PGB_CUDA(cudaMemcpyAsync(d1.p, nd.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(d1.p, inrm, KE);
      } else {
        lambda_out = lam_phys;
      }
    }
    scal(nd.p, 1.0 / norm(nd.p), KE);
    PGB_CUDA(cudaMemcpyAsync(delta_out, nd.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    sync();
  }
  g_stats.lambda = lambda_out;
  return lambda_out;
}

template <typename R>
void run_lin_eliash(const LinEliashArgs& a) {
  Inputs in;
  upload_inputs(in, a.kmap, a.invk, a.olist, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Smat, a.Cmat,
                nullptr, nullptr, a.uni);
  const long long KE = in.g.K * a.Norb * a.Norb, KC = in.g.K * a.Nchi * a.Nchi;
  DBuf<double> prt(a.Norb), init(a.Nk * a.Norb);
  prt.upload(a.prt, a.Norb);
  init.upload(a.init_delta, a.Nk * a.Norb);
  DBuf<double2> G(KE), D(KE);
  G.upload(a.Gk, KE);
  DBuf<cx<R>> chi(KC);
  {
    DBuf<double2> tmp(KC);
    tmp.upload(a.chi, KC);
    if (std::is_same<R, double>::value)
      PGB_CUDA(cudaMemcpyAsync(chi.p, tmp.p, KC * sizeof(double2), cudaMemcpyDeviceToDevice, ctx().stream));
    else narrow<R>(chi.p, tmp.p, KC);
  }
  EliashParams prm{a.temp, a.eps, a.itemax, a.gap_sym, a.arnoldi_m};
  *a.lambda_out = eliash_core<R>(in, chi.p, G.p, init.p, prt.p, prm, D.p, a.clobber_chi ? a.chi : nullptr);
  D.download(a.delta, KE);
  sync();
}

// ============================================================== pipeline ==
// FLEX self-energy -> G -> chi0 -> linearized Eliashberg, device resident
// between the stages (the reference's calc_lin_eliashberg_eq with
// sw_self=True, libs/plibs/_calc.py:370-405, as one call).
// Coarse-mesh warm start: the same model on the k mesh divided by
// coarse_kdiv (each axis that it divides) with Nw / coarse_wdiv frequencies,
// solved on FP32 bulk down to the FP32 rounding floor; its Sigma is
// interpolated to the fine mesh (sigma_interp) and its mu seeds the fine loop.
// H, its eigenvalues and eigenvectors on the coarse mesh are those of the fine
// mesh at the same k (transposed / conjugated at -k), so no hopping data is
// needed.
// Band data of one mesh on the host, in the C-ABI layouts (H, U: (No,No,Nk), e: (No,Nk))
struct HostBands {
  const double2* hamk;
  const double2* uni;
  const double* eig;
};

// Sigma seed of the fine problem `in` from the same model solved on the mesh
// and Matsubara set divided by (kdiv, wdiv), FP32 bulk down to its rounding
// floor.  While the coarse problem is itself large (>= 8 points per divided
// axis and >= 128 frequencies after another division), its own solve starts
// from a seed made the same way one level further down.
void coarse_seed_level(Inputs& in, const HostBands& hb, int64_t kdiv, int64_t wdiv, const FlexParams& prm,
                       DBuf<double2>& seed, double* mu_seed, int depth) {
  const Geom& g = in.g;
  const int No = in.Norb;
  auto div = [&](int n) { return (kdiv > 1 && n % kdiv == 0 && n / kdiv >= 2) ? n / (int)kdiv : n; };
  const int Nxc = div(g.Nx), Nyc = div(g.Ny), Nzc = g.Nz > 1 ? div(g.Nz) : 1;
  const int Nwc = std::max(1, g.Nw / (int)std::max<int64_t>(1, wdiv));
  std::vector<int64_t> kmap_c, invk_c;
  const int64_t Nkc = make_irr_mesh(Nxc, Nyc, Nzc, kmap_c, invk_c);
  Inputs ic;
  ic.Norb = No;
  ic.Nchi = in.Nchi;
  ic.Nk = (int)Nkc;
  ic.Nw = Nwc;
  build_geom(ic.g, kmap_c.data(), invk_c.data(), Nxc, Nyc, Nzc, Nkc, Nwc, No, in.Nchi);
  ic.p = in.p;
  const int fx = g.Nx / Nxc, fy = g.Ny / Nyc, fz = g.Nz / Nzc;
  std::vector<double2> hc((size_t)No * No * Nkc), uc((size_t)No * No * Nkc);
  std::vector<double> ec((size_t)No * Nkc);
  for (int64_t j = 0; j < Nkc; ++j) {
    const long long gc = ic.g.h_irr_grid[j];
    const long long x = gc % Nxc, y = (gc / Nxc) % Nyc, z = gc / ((long long)Nxc * Nyc);
    const long long gf = fx * x + (long long)g.Nx * (fy * y + (long long)g.Ny * fz * z);
    const int kf = g.h_grid_irr[gf], fl = g.h_grid_flag[gf];
    for (int e = 0; e < No * No; ++e) {
      const double2 h = hb.hamk[e + (size_t)No * No * kf], u = hb.uni[e + (size_t)No * No * kf];
      hc[e + (size_t)No * No * j] = fl ? conj(h) : h;  // H(-k) = H(k)^* under time reversal
      uc[e + (size_t)No * No * j] = fl ? conj(u) : u;
    }
    for (int n = 0; n < No; ++n) ec[n + (size_t)No * j] = hb.eig[n + (size_t)No * kf];
  }
  ic.H.alloc(hc.size());
  ic.H.upload(hc.data(), hc.size());
  ic.uni.alloc(uc.size());
  ic.uni.upload(uc.data(), uc.size());
  ic.eig.alloc(ec.size());
  ic.eig.upload(ec.data(), ec.size());
  ic.S.alloc((size_t)in.Nchi * in.Nchi);
  ic.C.alloc((size_t)in.Nchi * in.Nchi);
  PGB_CUDA(cudaMemcpyAsync(ic.S.p, in.S.p, sizeof(double) * in.Nchi * in.Nchi, cudaMemcpyDeviceToDevice,
                           ctx().stream));
  PGB_CUDA(cudaMemcpyAsync(ic.C.p, in.C.p, sizeof(double) * in.Nchi * in.Nchi, cudaMemcpyDeviceToDevice,
                           ctx().stream));
  FlexParams pc = prm;
  pc.eps = prm.eps;
  pc.stop_at_fp32_floor = true;
  // one level further down while the coarse problem is still large
  DBuf<double2> seed_c;
  double mu_cc = 0.0;
  const bool nest = depth < 1 && kdiv > 1 && Nxc / kdiv >= 8 && Nyc / kdiv >= 8 && Nwc / std::max<int64_t>(1, wdiv) >= 128;
  int iters_below = 0;
  if (nest) {
    const HostBands hbc{hc.data(), uc.data(), ec.data()};
    coarse_seed_level(ic, hbc, kdiv, wdiv, prm, seed_c, &mu_cc, depth + 1);
    iters_below = g_stats.iterations_coarse;
  }
  DBuf<double2> sc((size_t)ic.g.K * No * No);
  double mu_c = 0;
  log("[FLEX] warm start on the %dx%dx%d mesh with %d frequencies\n", Nxc, Nyc, Nzc, Nwc);
  mkself_core(ic, pc, sc.p, &mu_c, nest ? seed_c.p : nullptr, mu_cc, mu_cc, kPrecMixed);
  g_stats.iterations_coarse = g_stats.iterations + iters_below;
  g_stats.iterations = g_stats.iterations32 = 0;
  seed.alloc((size_t)g.K * No * No);
  sigma_interp(ic.g, g, sc.p, seed.p, No, prm.temp);
  *mu_seed = mu_c;
}

void coarse_seed(Inputs& in, const PipelineArgs& a, const FlexParams& prm, DBuf<double2>& seed, double* mu_seed) {
  const HostBands hb{a.hamk, a.uni, a.eig};
  coarse_seed_level(in, hb, a.coarse_kdiv, a.coarse_wdiv, prm, seed, mu_seed, 0);
}

template <typename R>
void run_pipeline_impl(const PipelineArgs& a, int prec) {
  g_stats = LastStats{};
  cudaStream_t st = ctx().stream;
  Timer t;
  t.start();
  Inputs in;
  upload_inputs(in, a.kmap, a.invk, a.olist, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Smat, a.Cmat,
                a.hamk, a.eig, a.uni);
  const long long K = in.g.K, KE = K * a.Norb * a.Norb, KC = K * a.Nchi * a.Nchi;
  DBuf<double> prt(a.Norb), init(a.Nk * a.Norb);
  prt.upload(a.prt, a.Norb);
  init.upload(a.init_delta, a.Nk * a.Norb);
  DBuf<double2> seed;
  if (a.sigma_seed) {
    require_finite(a.sigma_seed, (size_t)KE, "the Sigma seed");
    seed.alloc(KE);
    seed.upload(a.sigma_seed, KE);
  }
  const double t_h2d = t.stop();
  t.start();
  FlexParams prm{a.mu_init, a.fill, a.temp, a.scf_loop, a.pp, a.eps, a.sub_sigma, false, false, a.m_diis,
                 a.sw_rescale, a.sw_tail, 1.0};
  double seed_mu = a.seed_mu, seed_mu_old = a.seed_mu_old;
  const bool warm = !a.sigma_seed && (a.coarse_kdiv > 1 || a.coarse_wdiv > 1);
  if (warm) {
    Timer tw;
    tw.start();
    coarse_seed(in, a, prm, seed, &seed_mu);
    seed_mu_old = seed_mu;
    g_stats.t_warm = tw.stop();
  }
  DBuf<double2> sig(KE), G(KE), D(KE);
  double mu = 0;
  mkself_core(in, prm, sig.p, &mu, seed.p, seed_mu, seed_mu_old, prec);
  const int iters = g_stats.iterations;
  seed.release();
  PGB_CHECK(dyson(G.p, sig.p, in.H.p, mu, a.temp, in.Nk, in.Nw, in.Norb), "singular G^-1 in the Dyson step");
  double stoner_v = 0;
  {
    DBuf<cx<R>> chi(KC);
    TailRef tr{in.eig.p, in.uni.p, mu};
    chi0<R>(in.g, in.p, G.p, a.temp, a.sw_tail ? &tr : nullptr, chi.p);
    double cdw = 0;
    int qs = 0, qc = 0;
    stoner<R>(in.g, chi.p, in.S.p, in.C.p, &stoner_v, &cdw, &qs, &qc);
    ckchi_print(in.g, stoner_v, cdw, qs, qc);
    EliashParams ep{a.temp, a.eps_eliash, a.itemax, a.gap_sym, a.arnoldi_m};
    *a.lambda_out = eliash_core<R>(in, chi.p, G.p, init.p, prt.p, ep, D.p, nullptr);
  }
  g_stats.iterations = iters;
  const double t_compute = t.stop();
  t.start();
  sig.download(a.sigmak, KE);
  D.download(a.delta, KE);
  sync();
  const double t_d2h = t.stop();
  *a.mu_out = mu;
  *a.stoner_out = stoner_v;
  if (a.times_ms) {
    a.times_ms[0] = t_h2d;
    a.times_ms[1] = t_compute;
    a.times_ms[2] = t_d2h;
  }
  g_stats.mu = mu;
}

template void run_lin_eliash<float>(const LinEliashArgs&);
template void run_lin_eliash<double>(const LinEliashArgs&);
// ================================================ nonlinear Eliashberg ==
namespace {
// max |a - b| (b may be null: max |a|), two-level
__global__ void k_maxabs(double* part, const double2* a, const double2* b, long long n) {
  __shared__ double red[256];
  double m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = b ? a[i] - b[i] : a[i];
    m = fmax(m, hypot(v.x, v.y));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
double maxabs(const double2* a, const double2* b, long long n) {
  DBuf<double> part(1024), out(1);
  k_maxabs<<<1024, 256, 0, ctx().stream>>>(part.p, a, b, n);
  launch_check("maxabs");
  k_max_parts<<<1, 256, 0, ctx().stream>>>(out.p, part.p, 1024);
  launch_check("max_parts");
  ctx().kernel_launches += 2;
  double h = 0;
  out.download(&h, 1);
  sync();
  return h;
}
}  // namespace

void nonlin_bubbles(double2* xs_out, double2* xc_out, const double2* Gk, const double2* Fk, const double* Smat,
                    const double* Cmat, const int64_t* olist, const double* prt_host, const int64_t* kmap,
                    const int64_t* invk, double temp, int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Nchi,
                    int64_t Norb, int64_t Nx, int64_t Ny, int64_t Nz, bool singlet, bool vertex) {
  PGB_CHECK(Norb <= kMaxOrb, "Norb above the engine limit of 8 orbitals");
  Inputs in;
  upload_inputs(in, kmap, invk, olist, Nx, Ny, Nz, Nkall, Nk, Nw, Norb, Nchi, Smat, Cmat, nullptr, nullptr, nullptr);
  const Geom& g = in.g;
  const long long KE = g.K * Norb * Norb, KC = g.K * Nchi * Nchi;
  std::vector<double> hprt(prt_host, prt_host + Norb);
  DBuf<double2> G(KE), F(KE), XS(KC), XC(KC);
  G.upload(Gk, KE);
  F.upload(Fk, KE);
  chi0<double>(g, in.p, G.p, temp, nullptr, XS.p);
  chi0_ff<double>(g, in.p, F.p, hprt, temp, singlet, XC.p);
  combine_sc(XS.p, XC.p, KC);
  if (vertex) PGB_CHECK(vertex_sc(XS.p, XC.p, g.K, (int)Nchi, in.S.p, in.C.p, singlet), "zgesv failed in the SC vertex");
  XS.download(xs_out, KC);
  XC.download(xc_out, KC);
  sync();
}

void run_nonlin_eliash(const NonlinArgs& a) {
  g_stats = LastStats{};
  PGB_CHECK(a.Norb <= kMaxOrb, "Norb above the engine limit of 8 orbitals");
  cudaStream_t st = ctx().stream;
  Inputs in;
  upload_inputs(in, a.kmap, a.invk, a.olist, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Smat, a.Cmat,
                a.hamk, nullptr, nullptr);
  const Geom& g = in.g;
  const int No = (int)a.Norb, Nchi = (int)a.Nchi, Nk = (int)a.Nk, Nw = (int)a.Nw;
  const long long K = g.K, KE = K * No * No, KC = K * Nchi * Nchi;
  const bool singlet = a.gap_sym >= 0;
  const int m_eff = (int)std::max<int64_t>(a.m_diis, 1);
  const double pp = 0.3, eps_reg = 1.0e-12, weight = a.temp / (double)g.Nkall, scale = weight / (double)g.P;
  std::vector<double> hprt(a.prt, a.prt + No);
  DBuf<double> prt(No);
  prt.upload(a.prt, No);
  DBuf<double2> D(KE), ND(KE), Sig(KE), G(KE), G0(KE), F(KE), v0(KE), XS(KC), XC(KC);
  D.upload(a.delta, KE);
  G.upload(a.Gk, KE);
  std::vector<DBuf<double2>> xout(m_eff), res(m_eff);
  for (int i = 0; i < m_eff; ++i) {
    xout[i].alloc(KE);
    res[i].alloc(KE);
  }
  log(singlet ? "singlet\n" : "triplet\n");
  if (a.m_diis <= 1) log("DIIS disabled (m_diis=%lld); pure linear mixing pp=%4.2f.\n", (long long)a.m_diis, pp);
  else log("DIIS enabled, m_diis=%d; linear-mixing fallback pp=%4.2f.\n", m_eff, pp);
  auto norm2 = [&](const double2* x) { return dot_re(x, x, KE); };
  auto set_scaled = [&](double2* y, double c, const double2* x) {  // y = c x
    const double2* xs[1] = {x};
    const double2 cs[1] = {make_double2(c, 0.0)};
    lincomb(y, xs, cs, 1, KE);
  };
  auto chi_sc = [&]() {  // XS = chi0_S, XC = chi0_C (ffeliash.f90:454-489)
    chi0<double>(g, in.p, G.p, a.temp, nullptr, XS.p);
    chi0_ff<double>(g, in.p, F.p, hprt, a.temp, singlet, XC.p);
    combine_sc(XS.p, XC.p, KC);
    if (ctx().verbose) {  // the Stoner check only prints
      double sdw = 0, cdw = 0;
      int qs = 0, qc = 0;
      stoner<double>(g, XS.p, in.S.p, in.C.p, &sdw, &cdw, &qs, &qc);
      ckchi_print(g, sdw, cdw, qs, qc);
    }
    PGB_CHECK(vertex_sc(XS.p, XC.p, K, Nchi, in.S.p, in.C.p, singlet), "zgesv failed in the SC vertex");
  };
  int n_hist = 0, i_hist = 0, amp_phase = 1, npts = 0, n_polish = 0, n_anchor = 0;
  double a1 = 0, a2 = 0, g1 = 0, g2 = 0;
  double a_cur = std::sqrt(norm2(D.p)) + 1.0e-300;
  set_scaled(v0.p, 1.0 / a_cur, D.p);
  if (!a.sw_amp_newton) amp_phase = 2;
  PGB_CUDA(cudaMemcpyAsync(G0.p, G.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  const double delta0_max = maxabs(D.p, nullptr, KE) + 1.0e-30;
  if (a.sw_Vconst) {
    F.zero();
    chi_sc();
    mkfk(F.p, G.p, D.p, K, No);
  } else {
    mkfk(F.p, G.p, D.p, K, No);
    chi_sc();
  }
  if (!a.sw_sigma) Sig.zero();
  DeltaKernelCache<double> cache;  // the transformed V_Delta stays valid while V is constant
  int it = 0;
  for (it = 1; it <= a.itemax; ++it) {
    log("iter=%5d\n", it);
    mkdelta<double>(g, in.p, F.p, XC.p, in.S.p, in.C.p, prt.p, singlet, scale, ND.p,
                    a.sw_Vconst ? &cache : nullptr);
    const double diff = maxabs(ND.p, D.p, KE), dn = maxabs(D.p, nullptr, KE) + 1.0e-30,
                 new_max = maxabs(ND.p, nullptr, KE);
    log("  |D_new-D|max=%12.4E  rel=%12.4E  |D_new|max=%12.4E\n", diff, diff / dn, new_max);
    g_stats.esterr = diff / dn;
    if (diff / dn < a.eps) {
      PGB_CUDA(cudaMemcpyAsync(D.p, ND.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      log("converged at iter=%5d\n", it);
      break;
    }
    if (a.gap_min > 0.0 && new_max < a.gap_min * delta0_max) {
      PGB_CUDA(cudaMemcpyAsync(D.p, ND.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      log("gap collapsed: |D_new|max=%12.4E < %12.4E (likely T >= Tc; no SC solution), stopping\n", new_max,
          a.gap_min * delta0_max);
      break;
    }
    if (a.sw_amp_newton && amp_phase == 2 && n_polish >= 10) {  // re-anchor the shape
      a_cur = std::sqrt(norm2(D.p)) + 1.0e-300;
      set_scaled(v0.p, 1.0 / a_cur, D.p);
      npts = 0;
      a1 = a2 = g1 = g2 = 0.0;
      amp_phase = 1;
      ++n_anchor;
      log("  re-anchor #%d: v0 <- relaxed shape, re-solving amplitude\n", n_anchor);
    }
    if (amp_phase == 1) {
      // v0-anchored amplitude: g(a) = <v0, M[a v0]>/a = lam0 - c a^2, root of g = 1
      const double g_cur = dot_re(v0.p, ND.p, KE) / a_cur;
      a2 = a1;
      g2 = g1;
      a1 = a_cur;
      g1 = g_cur;
      npts = std::min(npts + 1, 2);
      double a_nxt;
      if (npts >= 2 && std::fabs(a1 * a1 - a2 * a2) > 1.0e-30) {
        const double cfit = (g1 - g2) / (a2 * a2 - a1 * a1), lam0 = g1 + cfit * a1 * a1;
        if (cfit > 1.0e-12 && lam0 > 1.0) {
          a_nxt = std::sqrt((lam0 - 1.0) / cfit);
          a_nxt = std::min(std::max(a_nxt, 0.3 * a_cur), 3.0 * a_cur);
        } else {
          a_nxt = 0.5 * a_cur;
        }
      } else {
        a_nxt = std::fabs(g_cur - 1.0) < 0.2 ? 0.9 * a_cur : 0.6 * a_cur;
      }
      if (std::fabs(g_cur - 1.0) < 2.0e-2) {
        amp_phase = 2;
        a_nxt = a_cur;
        n_polish = 0;
        n_hist = i_hist = 0;
        log("  amplitude solved (g=%9.5f); DIIS shape polish\n", g_cur);
      }
      set_scaled(D.p, a_nxt, v0.p);
      a_cur = a_nxt;
    } else {
      i_hist = i_hist % m_eff + 1;
      n_hist = std::min(n_hist + 1, m_eff);
      const int n = n_hist, slot = i_hist - 1;
      PGB_CUDA(cudaMemcpyAsync(xout[slot].p, ND.p, KE * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      {
        const double2* xs[2] = {ND.p, D.p};
        const double2 cs[2] = {make_double2(1.0, 0.0), make_double2(-1.0, 0.0)};
        lincomb(res[slot].p, xs, cs, 2, KE);
      }
      bool do_pulay = n >= 2 && m_eff >= 2;
      std::vector<int> idx(n);
      std::vector<double> c(n + 1, 0.0);
      if (do_pulay) {
        for (int h = 1; h <= n; ++h) idx[h - 1] = ((i_hist - n + h - 1) % m_eff + m_eff) % m_eff;
        const int nn = n + 1;
        std::vector<double> B((size_t)nn * nn, 0.0);
        for (int i = 0; i < n; ++i) {
          for (int j = 0; j < n; ++j) B[i * nn + j] = dot_re(res[idx[i]].p, res[idx[j]].p, KE);
          B[i * nn + i] += eps_reg;
          B[i * nn + n] = B[n * nn + i] = 1.0;
        }
        c[n] = 1.0;
        if (!solve_real(B, c, nn)) {
          log("DIIS: dgesv failed, falling back to linear mixing pp=0.30.\n");
          do_pulay = false;
        }
      }
      if (do_pulay) {
        std::vector<const double2*> xs(n);
        std::vector<double2> cs(n);
        for (int h = 0; h < n; ++h) {
          xs[h] = xout[idx[h]].p;
          cs[h] = make_double2(c[h], 0.0);
        }
        lincomb(D.p, xs.data(), cs.data(), n, KE);
      } else {
        const double2* xs[2] = {ND.p, D.p};
        const double2 cs[2] = {make_double2(pp, 0.0), make_double2(1.0 - pp, 0.0)};
        lincomb(D.p, xs, cs, 2, KE);
      }
      ++n_polish;
    }
    if (a.sw_sigma) {  // FLEX self-energy and the dressed G0 (no HF subtraction here)
      sigma<double>(g, in.p, G.p, XS.p, in.S.p, in.C.p, a.temp, Sig.p);
      PGB_CHECK(dyson(G0.p, Sig.p, in.H.p, a.mu, a.temp, Nk, Nw, No), "singular G^-1 in the Dyson step");
    }
    mkgreliah(G.p, G0.p, F.p, D.p, K, No);
    mkfkeliash(F.p, G0.p, G.p, D.p, K, No);
    if (!a.sw_Vconst) chi_sc();
  }
  g_stats.iterations = std::min<int>(it, (int)a.itemax);
  D.download(a.delta, KE);
  Sig.download(a.sigmak, KE);
  G.download(a.Gk, KE);
  sync();
}

// ============================================================ spin-orbit ==
namespace {
// the maps of a full k list for build_full_mesh without a Geom: the
// reference's invk alone (full-mesh kernels that need no FFT)
void full_mesh_from_invk(FullMesh& fm, const int64_t* invk, int64_t Nkall, int64_t Nk) {
  std::vector<int> irr(Nkall), flag(Nkall), minus(Nkall);
  for (int64_t i = 0; i < Nkall; ++i) {
    irr[i] = (int)invk[3 * i] - 1;
    flag[i] = (int)invk[3 * i + 1];
    minus[i] = (int)invk[3 * i + 2] - 1;
    PGB_CHECK(irr[i] >= 0 && irr[i] < Nk, "invk(1,:) outside [1,Nk]");
    PGB_CHECK(flag[i] == 0 || flag[i] == 1, "invk(2,:) must be 0 or 1");
  }
  fm.Nkall = Nkall;
  fm.irr.alloc(Nkall);
  fm.irr.upload(irr.data(), Nkall);
  fm.flag.alloc(Nkall);
  fm.flag.upload(flag.data(), Nkall);
  fm.minus.alloc(Nkall);
  fm.minus.upload(minus.data(), Nkall);
}

void spin_map(Geom& g, const SocSpin& sp, int64_t Norb) {
  PGB_CHECK(Norb <= kMaxOrb, "Norb above the engine limit of 8 orbitals");
  for (int a = 0; a < Norb; ++a) {
    PGB_CHECK(sp.invs[a] >= 1 && sp.invs[a] <= Norb, "invs entry outside [1,Norb]");
    PGB_CHECK(sp.slist[a] == 1 || sp.slist[a] == -1, "slist entries must be +1 or -1");
    g.spin.inv[a] = (int)sp.invs[a] - 1;
    g.spin.sgn[a] = (int)sp.slist[a];
  }
  g.spin.on = 1;
}

void upload_soc(Inputs& in, const int64_t* kmap, const int64_t* invk, const int64_t* olist, const SocSpin& sp,
                int64_t Nx, int64_t Ny, int64_t Nz, int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Norb, int64_t Nchi,
                const double* Vmat, const double2* hamk, const double* eig, const double2* uni) {
  PGB_CHECK(Nchi == 4 || Nchi == 16, "the spin-orbit engine supports Nchi = 4 or 16 (2 or 4 spin-orbitals)");
  upload_inputs(in, kmap, invk, olist, Nx, Ny, Nz, Nkall, Nk, Nw, Norb, Nchi, Vmat, Vmat, hamk, eig, uni);
  build_pairs_soc(in.p, in.g, olist, (int)Norb, (int)Nchi, sp.invs, sp.slist);
  in.soc = true;
  const size_t n2 = (size_t)Nchi * Nchi;
  std::vector<double> neg(Vmat, Vmat + n2);
  for (auto& x : neg) x = -x;
  in.V.alloc(n2);
  in.V.upload(Vmat, n2);
  in.Vneg.alloc(n2);
  in.Vneg.upload(neg.data(), n2);
}
}  // namespace

void run_mkself_soc(const MkselfArgs& a, const SocSpin& sp) {
  g_stats = LastStats{};
  Inputs in;
  upload_soc(in, a.kmap, a.invk, a.olist, sp, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Smat, a.hamk,
             a.eig, a.uni);
  FlexParams prm{a.mu_init, a.fill, a.temp, a.scf_loop, a.pp, a.eps, a.sub_sigma, a.sw_out, a.sw_in, a.m_diis,
                 a.sw_rescale, false, a.sigma_scale};
  const long long KE = in.g.K * a.Norb * a.Norb;
  DBuf<double2> sig(KE);
  mkself_core(in, prm, sig.p, a.mu_out, nullptr, 0.0, 0.0, 64);
  sig.download(a.sigmak, KE);
  sync();
}

double run_chi0_soc(double2* chi_out, const double* Vmat, const double2* Gk, const int64_t* kmap,
                    const int64_t* invk, const int64_t* olist, const SocSpin& sp, double temp, int64_t Nx, int64_t Ny,
                    int64_t Nz, int64_t Nw, int64_t Nk, int64_t Nkall, int64_t Nchi, int64_t Norb) {
  g_stats = LastStats{};
  Inputs in;
  upload_soc(in, kmap, invk, olist, sp, Nx, Ny, Nz, Nkall, Nk, Nw, Norb, Nchi, Vmat, nullptr, nullptr, nullptr);
  const long long KE = in.g.K * Norb * Norb, KC = in.g.K * Nchi * Nchi;
  DBuf<double2> G(KE), chi(KC);
  G.upload(Gk, KE);
  chi0<double>(in.g, in.p, G.p, temp, nullptr, chi.p);
  double sdw = 0, cdw = 0;
  int qs = 0, qc = 0;
  stoner<double>(in.g, chi.p, in.Vneg.p, in.Vneg.p, &sdw, &cdw, &qs, &qc);
  ckchi_print_soc(in.g, sdw, qs);
  g_stats.stoner = sdw;
  chi.download(chi_out, KC);
  sync();
  return sdw;
}

void run_lin_eliash_soc(const LinEliashSocArgs& a) {
  g_stats = LastStats{};
  cudaStream_t st = ctx().stream;
  Inputs in;
  upload_soc(in, a.kmap, a.invk, a.olist, a.sp, a.Nx, a.Ny, a.Nz, a.Nkall, a.Nk, a.Nw, a.Norb, a.Nchi, a.Vmat, nullptr,
             nullptr, a.uni);
  const Geom& g = in.g;
  FullMesh fm;
  build_full_mesh(fm, g, a.invk);
  const int No = (int)a.Norb, Nchi = (int)a.Nchi;
  const long long KE = g.K * No * No, KC = g.K * Nchi * Nchi, KF = fm.Nkall * g.Nw * No * No;
  const int gap_sym = (int)a.gap_sym;
  DBuf<double2> chi(KC), G(KE), F(KF), D(KF);
  chi.upload(a.chi, KC);
  {
    Timer tv;
    tv.start();
    PGB_CHECK(vertex_soc(chi.p, g.K, Nchi, in.V.p), "zgesv failed in V_delta");  // chi -> V_Delta
    g_stats.t_vertex += tv.stop();
  }
  chi.download(a.chi, KC);
  G.upload(a.Gk, KE);
  DBuf<double> init((size_t)a.Nk * No), ones(fm.Nkall);
  init.upload(a.init_delta, (size_t)a.Nk * No);
  {
    std::vector<double> h1(fm.Nkall, 1.0);
    ones.upload(h1.data(), fm.Nkall);
  }
  std::vector<double> hV(a.Vmat, a.Vmat + (size_t)Nchi * Nchi);
  std::vector<int> invschi(Nchi);
  for (int l = 0; l < Nchi; ++l) invschi[l] = (int)a.invschi[l];
  const double scale = -a.temp / (double)g.Nkall;  // A v = -(T/Nkall) mkdelta_soc(mkfk_soc(v))
  Timer ta;
  auto apply_op = [&](double2* out, const double2* v) {
    ta.start();
    mkfk_soc(F.p, G.p, v, fm, g, gap_sym);
    mkdelta_soc(g, in.p, fm, F.p, chi.p, hV, invschi, gap_sym, scale, out);
    g_stats.t_apply += ta.stop();
    g_stats.applies += 1;
  };
  const int Nkf = (int)fm.Nkall;
  auto inner = [&](const double2* u, const double2* v) {  // 2 sum conj(u) v (feliashwithsoc.f90:400-424)
    const double2 s = inner_w(u, v, ones.p, Nkf, KF);
    return make_double2(2.0 * s.x, 2.0 * s.y);
  };
  auto norm = [&](const double2* f) { return std::sqrt(2.0 * inner_w(f, f, ones.p, Nkf, KF).x); };
  auto init_vec = [&](double2* d) {
    initial_delta_soc(d, init.p, in.uni.p, fm, g, gap_sym);
    const double n2 = inner_w(d, d, ones.p, Nkf, KF).x;
    PGB_CHECK(n2 > 0, "Error: get_initial_delta_soc norm <= 0");
    scal(d, 1.0 / std::sqrt(2.0 * n2), KF);
  };
  double lam = 0.0;
  if (a.arnoldi_m > 0) {
    lam = arnoldi_two_pass((int)a.arnoldi_m, KF, apply_op, inner, norm, init_vec, D.p);
  } else {
    // shifted power method of lin_eliash_soc (feliashwithsoc.f90:60-110): pass 2
    // runs with the shift |newdelta| of pass 1 and no deflation
    DBuf<double2> nd(KF), tmp(KF);
    double norm2 = 0.0, nrm = 1.0;
    for (int i_eig = 1; i_eig <= 2; ++i_eig) {
      init_vec(D.p);
      int count = 0;
      for (int it = 1; it <= a.itemax; ++it) {
        apply_op(nd.p, D.p);
        if (norm2 != 0.0) axpy(nd.p, make_double2(norm2, 0), D.p, KF);
        nrm = norm(nd.p);
        PGB_CHECK(nrm > 0, "Error: norm <= 0 in iter_loop");
        const double inrm = 1.0 / nrm;
        const double lam_rq = inner(D.p, nd.p).x;
        PGB_CUDA(cudaMemcpyAsync(tmp.p, nd.p, KF * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(tmp.p, inrm, KF);
        axpy(tmp.p, make_double2(-1, 0), D.p, KF);
        const double ep = norm(tmp.p);
        axpy(tmp.p, make_double2(2, 0), D.p, KF);
        const double en = norm(tmp.p);
        const double verr = std::min(ep, en);
        lam = lam_rq - norm2;
        log("%3d lambda_elsh=%16.8E\n", it, lam);
        if (verr < a.eps) {
          if (lam > 0.1 || lam < 0.0) break;
          if (verr < a.eps * 1.0e-2) ++count;
          if (count > 30) break;
        }
        PGB_CUDA(cudaMemcpyAsync(D.p, nd.p, KF * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        scal(D.p, inrm, KF);
      }
      log(" eliash= %.15g\n", lam);
      if (i_eig == 1 && lam > 0.0) break;
      norm2 = nrm;
    }
    PGB_CUDA(cudaMemcpyAsync(D.p, nd.p, KF * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    scal(D.p, 1.0 / norm(D.p), KF);
  }
  g_stats.lambda = lam;
  D.download(a.delta, KF);
  sync();
}

void run_mkfk_soc(double2* fk, const double2* Gk, const double2* delta, const int64_t* invk, const SocSpin& sp,
                  int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Norb, int64_t gap_sym) {
  Geom g;
  g.Nk = (int)Nk;
  g.Nw = (int)Nw;
  g.Norb = (int)Norb;
  spin_map(g, sp, Norb);
  FullMesh fm;
  full_mesh_from_invk(fm, invk, Nkall, Nk);
  const long long KE = Nk * Nw * Norb * Norb, KF = Nkall * Nw * Norb * Norb;
  DBuf<double2> G(KE), D(KF), F(KF);
  G.upload(Gk, KE);
  D.upload(delta, KF);
  mkfk_soc(F.p, G.p, D.p, fm, g, (int)gap_sym);
  F.download(fk, KF);
  sync();
}

void run_orb_to_band_soc(double2* deltab, const double2* delta, const double2* uni, const int64_t* invk,
                         const SocSpin& sp, int64_t Norb, int64_t Nkall, int64_t Nk, int64_t Nw) {
  Geom g;
  g.Nk = (int)Nk;
  g.Nw = (int)Nw;
  g.Norb = (int)Norb;
  spin_map(g, sp, Norb);
  FullMesh fm;
  full_mesh_from_invk(fm, invk, Nkall, Nk);
  const long long KF = Nkall * Nw * Norb * Norb, KU = Nk * Norb * Norb, KB = Nkall * Norb * Norb;
  DBuf<double2> D(KF), U(KU), B(KB);
  D.upload(delta, KF);
  U.upload(uni, KU);
  orb_to_band_soc(B.p, D.p, U.p, fm, g);
  B.download(deltab, KB);
  sync();
}

void run_chis_chic_soc(double2* chic, double2* chiszz, double2* chispm, const double2* chi, const double* Vmat,
                       const int64_t* orb_list, const int64_t* olist, const int64_t* slist, int64_t Nk, int64_t Nw,
                       int64_t Nchi, int64_t Norb) {
  PGB_CHECK(Nchi % 4 == 0, "Nchi must be a multiple of 4 for the spin-orbit channels");
  const long long K = Nk * Nw, KC = K * Nchi * Nchi;
  std::vector<int> o1(Nchi), o2(Nchi), sl(Norb), ol(Nchi);
  for (int64_t l = 0; l < Nchi; ++l) {
    o1[l] = (int)olist[l] - 1;
    o2[l] = (int)olist[Nchi + l] - 1;
    PGB_CHECK(o1[l] >= 0 && o1[l] < Norb && o2[l] >= 0 && o2[l] < Norb, "olist entry outside [1,Norb]");
    ol[l] = (int)orb_list[l];
  }
  for (int64_t a = 0; a < Norb; ++a) sl[a] = (int)slist[a];
  DBuf<double2> X(KC);
  DBuf<double> V((size_t)Nchi * Nchi);
  X.upload(chi, KC);
  V.upload(Vmat, (size_t)Nchi * Nchi);
  chis_chic_soc(chic, chiszz, chispm, X.p, K, (int)Nk, (int)Nchi, V.p, o1, o2, sl, ol);
}

// Eliashberg-stage bulk (final chi0, V_Delta, Arnoldi applies): FP32 in the
// FP32 mode or with PYRPA_GB_ELIASH=fp32; double-float in the mixed mode
// unless PYRPA_GB_ELIASH=fp64 (df64: double-float with the FP64 V_Delta
// solve); FP64 otherwise.  With FP32 bulk there, lambda of the 5-orbital
// 64x64x2048 model moved by 3.6e-6 relative.
void run_pipeline(const PipelineArgs& a, int prec) {
  const char* e = std::getenv("PYRPA_GB_ELIASH");
  const std::string ev = e ? e : "";
  if (prec == 32 || ev == "fp32") run_pipeline_impl<float>(a, prec);
  else if (prec == kPrecMixed && ev != "fp64") run_pipeline_impl<dfl>(a, prec);  // "df64": FP64 V_Delta solve
  else run_pipeline_impl<double>(a, prec);
}

}  // namespace pgb
