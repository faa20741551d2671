// Argument bundles of the two solver drivers (host pointers as the C ABI
// receives them) and the statistics of the last solve.
#pragma once

#include <cstdint>
#include <vector>

#include "flex.cuh"

namespace pgb {

struct MkselfArgs {
  double2* sigmak;                 // out (Nk,Nw,Norb,Norb)
  double* mu_out;
  const double *Smat, *Cmat;       // (Nchi,Nchi)
  const int64_t *kmap, *invk, *olist;
  const double2* hamk;             // (Norb,Norb,Nk)
  const double* eig;               // (Norb,Nk)
  const double2* uni;              // (Norb,Norb,Nk)
  double mu_init, fill, temp;
  int64_t scf_loop;
  double pp, eps;
  int64_t Nkall, Nk, Nw, Norb, Nchi, Nx, Ny, Nz, sub_sigma;
  bool sw_out, sw_in;
  int64_t m_diis;
  bool sw_rescale, sw_tail;
  double sigma_scale;
};

struct LinEliashArgs {
  double2* delta;                  // out (Nk,Nw,Norb,Norb)
  double2* chi;                    // in (Nk,Nw,Nchi,Nchi); overwritten with V_Delta
  const double2 *Gk, *uni;
  const double* init_delta;        // (Nk,Norb)
  const double *Smat, *Cmat;
  const int64_t* olist;
  const double* prt;
  const int64_t *kmap, *invk;
  double temp, eps;
  int64_t Nkall, Nk, Nw, Nchi, Norb, Nx, Ny, Nz, itemax, gap_sym, arnoldi_m;
  double* lambda_out;
  bool clobber_chi = true;
};

struct PipelineArgs {
  double2* sigmak;                 // out (Nk,Nw,Norb,Norb)
  double* mu_out;
  double2* delta;                  // out (Nk,Nw,Norb,Norb)
  double* lambda_out;
  double* stoner_out;
  double* times_ms;                // out [3]: H2D, device compute, D2H (CUDA events); may be null
  const double *Smat, *Cmat;
  const int64_t *kmap, *invk, *olist;
  const double2* hamk;
  const double* eig;
  const double2* uni;
  const double* init_delta;        // (Nk,Norb)
  const double* prt;               // (Norb)
  const double2* sigma_seed;       // optional starting Sigma (Nk,Nw,Norb,Norb); null: G0 start
  double seed_mu, seed_mu_old;
  double mu_init, fill, temp;
  int64_t scf_loop;
  double pp, eps;
  int64_t Nkall, Nk, Nw, Norb, Nchi, Nx, Ny, Nz, sub_sigma, m_diis;
  bool sw_rescale, sw_tail;
  int64_t gap_sym, arnoldi_m, itemax;
  double eps_eliash;
  // coarse-mesh warm start: k mesh and Matsubara count divided by these
  // (1 = not coarsened; both 1 = no warm start)
  int64_t coarse_kdiv = 1, coarse_wdiv = 1;
};

// nonlinear FLEX-Eliashberg loop (ffeliash.f90:2-314), host pointers as the ABI receives them
struct NonlinArgs {
  double2* delta;                  // inout (Nk,Nw,Norb,Norb)
  double2* sigmak;                 // out
  double2* Gk;                     // inout: initial G, on exit the last SC G
  const double2* hamk;             // (Norb,Norb,Nk)
  const double *Smat, *Cmat;
  const int64_t* olist;
  const double* prt;
  const int64_t *kmap, *invk;
  double mu, temp, eps;
  int64_t Nkall, Nk, Nw, Nchi, Norb, Nx, Ny, Nz, itemax, gap_sym;
  bool sw_sigma, sw_Vconst;
  int64_t m_diis;
  double gap_min;
  bool sw_amp_newton;
};

// uploaded model data shared by the solvers
struct Inputs {
  Geom g;
  Pairs p;
  DBuf<double> S, C, eig;
  DBuf<double2> H, uni;
  int Norb = 1, Nchi = 1, Nk = 1, Nw = 1;
  // spin-orbit runs: V and -V (Fortran order); the pairs and g.spin carry the
  // spin partners (fselfwithsoc.f90)
  bool soc = false;
  DBuf<double> V, Vneg;
};

struct FlexParams {
  double mu_init, fill, temp;
  int64_t scf_loop;
  double pp, eps;
  int64_t sub_sigma;
  bool sw_out, sw_in;
  int64_t m_diis;
  bool sw_rescale, sw_tail;
  double sigma_scale;
  bool stop_at_fp32_floor = false;  // mixed schedule: stop where it would switch to FP64
};

struct EliashParams {
  double temp, eps;
  int64_t itemax, gap_sym, arnoldi_m;
};

struct LastStats {
  int iterations = 0, iterations32 = 0;  // FLEX iterations (of which on FP32 bulk)
  int iterations_finish32 = 0;           // mixed schedule: FP64 chi0/Sigma with FP32 vertex
  int iterations_coarse = 0;             // FLEX iterations of the coarse-mesh warm start
  double t_warm = 0;                     // device ms of the warm start (coarse solve + interpolation)
  double esterr = 0, stoner = 0, mu = 0, lambda = 0;
  int applies = 0;
  // milliseconds on the device (CUDA events on the library stream)
  double t_chi0 = 0, t_vertex = 0, t_sigma = 0, t_diis = 0, t_mu = 0, t_dyson = 0, t_apply = 0;
  double t_stoner = 0;  // Stoner factor (and the sw_rescale clamp) of the FLEX loop
  // real parts of the last Arnoldi pass's Ritz values on the operator's own
  // scale (the pass-2 shift undone), largest first
  double ritz[16] = {0};
  int nritz = 0;
  // residual |A x - lambda x| / |lambda| of the returned Ritz pair and the
  // Arnoldi cycles of the pass that produced it (restarts + 1)
  double ritz_residual = 0;
  int arnoldi_cycles = 0;
  int judge_polish = 0;  // mixed schedule: full judging steps taken after convergence
};

// bulk type of each stage of a FLEX iteration: 32 FP32, 64 FP64, 48 double-float
struct StagePrec {
  int chi0, vertex, sigma;
};

// precision schedule of the FLEX loop: 64, 32 or kPrecMixed
constexpr int kPrecMixed = 3264;
constexpr int kPrecDF = 48;  // double-float chi0 and Sigma convolutions, FP64 elsewhere
constexpr double kMixSwitch = 2.0e-3;  // residual at which the mixed schedule leaves FP32
constexpr int kMixStall = 6;           // or after this many FP32 iterations without a new minimum
constexpr double kMixStallFrom = 0.1;  //   counted once the residual has been below this
constexpr int kMidDfNu = 4;            // middle phase: bosonic frequencies with a double-float vertex
constexpr int kJudgePolish = 0;        // full judging steps after convergence (mixed schedule)
// mixed schedule, restarted Arnoldi of the double-float Eliashberg stage: its
// first cycles may run on an FP32 copy of the operator, at most this many
// (PYRPA_GB_ELIASH_FP32 sets it; 0, the default, runs every cycle in
// double-float), until the Ritz residual over lambda is below kEliashFp32Tol
constexpr int kEliashFp32Cycles = 0;
constexpr double kEliashFp32Tol = 1.0e-5;

// the reference's irreducible TRS mesh (generate_irr_kpoint_inv): kmap and
// invk (3 per full point), returns Nk
int64_t make_irr_mesh(int64_t nx, int64_t ny, int64_t nz, std::vector<int64_t>& kmap, std::vector<int64_t>& invk);

void run_mkself(const MkselfArgs& a, int prec);
template <typename R> void run_lin_eliash(const LinEliashArgs& a);
void run_pipeline(const PipelineArgs& a, int prec);
void run_nonlin_eliash(const NonlinArgs& a);

// ---- spin-orbit coupling (fselfwithsoc.f90, fchi0withsoc.f90, feliashwithsoc.f90)
struct SocSpin {
  const int64_t *invs, *slist;     // (Norb) 1-based spin partner, +-1 spin label
};
// mkself_soc: the FLEX loop in FP64 with Vmat in place of Smat (Cmat unused)
void run_mkself_soc(const MkselfArgs& a, const SocSpin& sp);
// get_chi0_soc: bubble (Nk,Nw,Nchi,Nchi) and its Stoner factor max Re eig(-chi0 V)
double run_chi0_soc(double2* chi_out, const double* Vmat, const double2* Gk, const int64_t* kmap,
                    const int64_t* invk, const int64_t* olist, const SocSpin& sp, double temp, int64_t Nx, int64_t Ny,
                    int64_t Nz, int64_t Nw, int64_t Nk, int64_t Nkall, int64_t Nchi, int64_t Norb);
struct LinEliashSocArgs {
  double2* delta;                  // out (Nkall,Nw,Norb,Norb)
  double2* chi;                    // in (Nk,Nw,Nchi,Nchi); overwritten with V_Delta
  const double2 *Gk, *uni;
  const double *init_delta, *Vmat;
  const int64_t *olist, *kmap, *invk, *invschi;
  SocSpin sp;
  double temp, eps;
  int64_t Nkall, Nk, Nw, Nchi, Norb, Nx, Ny, Nz, itemax, gap_sym, arnoldi_m;
};
void run_lin_eliash_soc(const LinEliashSocArgs& a);
void run_mkfk_soc(double2* fk, const double2* Gk, const double2* delta, const int64_t* invk, const SocSpin& sp,
                  int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Norb, int64_t gap_sym);
void run_orb_to_band_soc(double2* deltab, const double2* delta, const double2* uni, const int64_t* invk,
                         const SocSpin& sp, int64_t Norb, int64_t Nkall, int64_t Nk, int64_t Nw);
void run_chis_chic_soc(double2* chic, double2* chiszz, double2* chispm, const double2* chi, const double* Vmat,
                       const int64_t* orb_list, const int64_t* olist, const int64_t* slist, int64_t Nk, int64_t Nw,
                       int64_t Nchi, int64_t Norb);
// chi0_S / chi0_C of G and F (vertex: V_sigma / V_Delta instead), host arrays
void nonlin_bubbles(double2* xs_out, double2* xc_out, const double2* Gk, const double2* Fk, const double* Smat,
                    const double* Cmat, const int64_t* olist, const double* prt_host, const int64_t* kmap,
                    const int64_t* invk, double temp, int64_t Nkall, int64_t Nk, int64_t Nw, int64_t Nchi,
                    int64_t Norb, int64_t Nx, int64_t Ny, int64_t Nz, bool singlet, bool vertex);
const LastStats& last_stats();

}  // namespace pgb
