// GB300 FLEX / RPA / linearized-Eliashberg engine: geometry, orbital-pair
// tables and the stage drivers the C ABI (abi.cu) calls.
//
// Data layout in HBM.  Per-(k,iw) quantities keep the reference's Fortran
// layout so the C ABI copies them without reshuffling:
//   G, Sigma, Delta, F : (Nk, Nw, Norb, Norb) complex, k fastest
//   chi, V             : (Nk, Nw, Nchi, Nchi), k fastest
// The FFT work arrays are full-grid (x, y, z, t) arrays, x fastest, one
// P = Nkall*2Nw block per orbital element; the t axis of a transformed array
// may be stored digit-transposed (FFT4D position tables).
#pragma once

#include <cstdint>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "linalg.cuh"

namespace pgb {

// Time-reversal partner of each orbital: G_ab(-k, iw) = sgn_a sgn_b G_{inv b, inv a}(k, iw).
// Identity with sgn = +1 without spin-orbit coupling; with it, inv is the
// spin partner and sgn the spin label (fchi0withsoc.f90:63-78).
struct SpinMap {
  int inv[kMaxOrb];
  int sgn[kMaxOrb];
  int on;
};

struct Geom {
  SpinMap spin;
  int Nx = 1, Ny = 1, Nz = 1, Nw = 1, Nk = 1, Norb = 1, Nchi = 1;
  long long Nkall = 1, M = 2, P = 2, K = 1;
  std::vector<int> h_grid_irr, h_grid_flag, h_irr_grid;
  std::vector<double> h_kweight;
  std::vector<int64_t> h_kmap;  // 3 per full point, as passed (for progress prints)
  std::vector<int> h_full_of_grid;  // full-list index of each grid cell
  DBuf<int> grid_irr, grid_flag, irr_grid;
  DBuf<double> kweight;
};

// Builds the grid maps from the reference's kmap(3,Nkall) / invk(3,Nkall)
// (1-based irreducible index, 0/1 flag) and validates them.
void build_geom(Geom& g, const int64_t* kmap, const int64_t* invk, int64_t Nx, int64_t Ny,
                int64_t Nz, int64_t Nk, int64_t Nw, int64_t Norb, int64_t Nchi);

struct ChiPair {
  int l, m, m2, l2;  // irreducible (m,l) and exchange partner (m2,l2), 0-based
  int e13, e42;      // orbital elements a + Norb*b of G13 and G42
  int self;          // partner is the pair itself
  double2 J;         // tau=0 jump coefficient (tail reference only)
  int pneg;          // the partner is -conj instead of conj (spin-orbit sign)
};

struct Term {  // one (m,l) term of a sigma / delta contraction
  int m, l, ef;    // pair indices and the G/F element multiplied with it
};

struct Pairs {
  int Norb = 1, Nchi = 1;
  std::vector<int> o1, o2;                       // 0-based orbitals of chi index l
  std::vector<ChiPair> chi;                      // irreducible pairs for chi0
  std::vector<std::vector<Term>> sigma;          // per output element a + Norb*b
  std::vector<std::vector<Term>> delta;          // per output element a + Norb*b (a >= b)
};

// chi_map / irr_chi from olist (fchi.f90:421-481) or taken from the caller
// (get_chi0_conv_ passes them, 1-based, int32, Fortran layout).
void build_pairs(Pairs& p, const int64_t* olist, int Norb, int Nchi, const int32_t* irr_chi = nullptr,
                 const int32_t* chi_map = nullptr);
// spin-orbit variant: exchange map with spin flips (fchi0withsoc.f90:216-279),
// partner signs sgnsig2, and the spin map of g
void build_pairs_soc(Pairs& p, Geom& g, const int64_t* olist, int Norb, int Nchi, const int64_t* invs,
                     const int64_t* slist);

// ------------------------------------------------------------------ stages
// All pointers are device pointers; R is the bulk (FFT/contraction) type.

// Gk = G0 (fself.f90:1-41) from eig (Norb,Nk) and uni (Norb,Norb,Nk)
void green0(double2* G, const double* eig, const double2* uni, double mu, double temp, int Nk,
            int Nw, int Norb);
// Gk = (iw + mu - H - Sigma)^-1 (fself.f90:43-157); returns false if singular
bool dyson(double2* G, const double2* sig, const double2* hamk, double mu, double temp, int Nk,
           int Nw, int Norb);
void green_inv_only(double2* G, const double2* sig, const double2* hamk, double mu, double temp,
                    int Nk, int Nw, int Norb);
bool invert_blocks(double2* G, long long nmat, int Norb, long long stride_mat, long long stride_el);

struct TailRef {
  const double* eig = nullptr;   // (Norb, Nk)
  const double2* uni = nullptr;  // (Norb, Norb, Nk)
  double mu = 0;
};

// chi0 by FFT convolution (fchi.f90:508-635), optionally tail-corrected
// (fchi.f90:637-892).  chi (Nk,Nw,Nchi,Nchi) of type cx<R> is overwritten.
template <typename R>
void chi0(const Geom& g, const Pairs& p, const double2* G, double temp, const TailRef* tail,
          cx<R>* chi);
// Stoner factors: max Re eig(chi0(q,0) S) and of -chi0(q,0) C (fchi.f90:352-399)
template <typename R>
void stoner(const Geom& g, const cx<R>* chi, const double* S, const double* C, double* sdw,
            double* cdw, int* q_sdw, int* q_cdw);
// in-place vertex: mode 0 V_sigma (fUJ.f90:318-365), 1 singlet / 2 triplet
// V_Delta (fUJ.f90:253-316), 3 chi_s, 4 chi_c with nu=0 slices only
template <typename R>
bool vertex(cx<R>* chi, long long nmat, long long stride, int Nchi, const double* S, const double* C,
            int mode);
template <typename R> void scale_chi(cx<R>* chi, long long n, double s);
// Sigma by FFT convolution (fself.f90:159-285), thresholded, FP64 output
template <typename R>
void sigma(const Geom& g, const Pairs& p, const double2* G, const cx<R>* V, const double* S,
           const double* C, double temp, double2* sig);
void hf_subtract(double2* sig, int Nk, int Nw, int Norb, int mode);

// reductions (deterministic two-level)
double dot_re(const double2* a, const double2* b, long long n);
double2 inner_w(const double2* a, const double2* b, const double* kw, int Nk, long long n);
double filling(const double2* eig_g, const double* eig, int Nk, int Nw, int Norb, double mu,
               double temp);
bool eig_gkinv(double2* eig_g, const double2* hamk, const double2* sig, int Nk, int Nw, int Norb);
// coefficients of det(z - H - Sigma) per (k, iw) and the filling from them
void charpoly_gk(double2* cp, const double2* hamk, const double2* sig, int Nk, int Nw, int Norb);
double filling_cp(const double2* cp, const double* eig, int Nk, int Nw, int Norb, double mu, double temp);

// Eliashberg
void mkfk(double2* F, const double2* G, const double2* D, long long K, int Norb);
// Transformed pairing vertex of every mkdelta term, kept across Arnoldi steps
// when it fits in HBM (the reference re-transforms it on every application).
template <typename R> struct DeltaKernelCache {
  bool built = false;
  DBuf<cx<R>> W;
  std::vector<long long> offset;  // first term of each output element
  // the one-launch contraction: outputs with terms, their terms' F element
  // and the first term of each (device)
  std::vector<int> out_elems;
  DBuf<int> ef, tb;
};
// Fbulk: F already in the bulk type (then F is not read; the parity factors
// prt must be +-1)
template <typename R>
void mkdelta(const Geom& g, const Pairs& p, const double2* F, const cx<R>* Vd, const double* S,
             const double* C, const double* prt, bool singlet, double scale, double2* out,
             DeltaKernelCache<R>* cache, const cx<R>* Fbulk = nullptr);
// F = -(G Delta) G^H in double-float (Norb <= 5; false otherwise)
bool mkfk_df(cdf* F, const cdf* G, const double2* D, long long K, int Norb);
void hermitize(double2* D, long long K, int Norb);
void initial_delta(double2* D, const double* init, const double2* uni, int Nk, int Nw, int Norb,
                   int gap_sym);
void axpy(double2* y, double2 a, const double2* x, long long n);         // y += a x
void scal(double2* y, double a, long long n);
void lincomb(double2* y, const double2* const* xs, const double2* cs, int m, long long n);

// Seed for a fine-mesh FLEX solve from a coarse-mesh one: Sigma on the coarse
// irreducible mesh gc (Nw_c frequencies) is Fourier-interpolated in k to the
// fine mesh gf (zero padding of Sigma(R), the Nyquist planes split in half) and
// extended from Nw_c to Nw_f frequencies with the tail c0 + c1/(i w) through
// two interior frequencies.  Both meshes share T; coarse k points must lie on
// the fine mesh (Nx_f a multiple of Nx_c, and so on).
void sigma_interp(const Geom& gc, const Geom& gf, const double2* sig_c, double2* sig_f, int Norb, double temp);

// Sigma (Nk, Nw_old, Norb, Norb) of the mesh at temp_old onto Nw_new
// frequencies at temp_new (plibs.regrid_sigma_bin, libs/plibs/_calc.py:52-182)
void regrid_sigma(double2* out, const double2* sig, int Nk, int Nw_old, int Nw_new, int Norb, double temp_old,
                  double temp_new, double w_scale);

// Sigma or Delta on the irreducible k points (or the full grid) -> R space for
// the first Ncut frequencies, [Norb][Norb][Ncut][z][y][x] (plibs Wannier writers)
void wannier_r(double2* out, const double2* data, const Geom& g, int Nw, int No, int Ncut, bool full_bz);

// nonlinear FLEX-Eliashberg (ffeliash.f90): SC Dyson updates, chi^FF bubble,
// chi0_S/chi0_C, and the two-channel vertex (V_sigma into XS, V_Delta into XC)
void mkgreliah(double2* G, const double2* G0, const double2* F, const double2* D, long long K, int Norb);
void mkfkeliash(double2* F, const double2* G0, const double2* G, const double2* D, long long K, int Norb);
template <typename R>
void chi0_ff(const Geom& g, const Pairs& p, const double2* F, const std::vector<double>& prt, double temp,
             bool singlet, cx<R>* chi);
void combine_sc(double2* gg, double2* ff, long long n);
bool vertex_sc(double2* XS, double2* XC, long long K, int Nchi, const double* S, const double* C, bool singlet);

// small host helpers
void ckchi_print(const Geom& g, double sdw, double cdw, int qs, int qc);
void ckchi_print_soc(const Geom& g, double v, int q);
template <typename R> void widen(double2* out, const cx<R>* in, long long n);
// out = in between any two bulk types (float, double, double-float)
template <typename To, typename From> void convert(cx<To>* out, const cx<From>* in, long long n);
template <typename R> void narrow(cx<R>* out, const double2* in, long long n);


// ---------------------------------------------------- spin-orbit coupling --
// Maps of the reference's full k list (kmap/invk order): irreducible index,
// direct/TRS flag, index of -k, and mesh cell, per full index; full index per cell.
struct FullMesh {
  long long Nkall = 0;
  DBuf<int> irr, flag, minus, grid, full;
};
void build_full_mesh(FullMesh& fm, const Geom& g, const int64_t* invk);
// -V (I + chi0 V)^-1 in place on (K, Nchi, Nchi) matrices; false on a singular matrix
bool vertex_soc(double2* chi, long long K, int Nchi, const double* V);
// nu = 0 channel sums of get_chis_chic_soc into host arrays (Nk, Nchi/4, Nchi/4)
void chis_chic_soc(double2* chic, double2* chiszz, double2* chispm, const double2* chi, long long K, int Nk, int Nchi,
                   const double* V, const std::vector<int>& o1, const std::vector<int>& o2,
                   const std::vector<int>& slist, const std::vector<int>& orb_list);
// full-mesh anomalous Green function (mkfk_trs_soc)
void mkfk_soc(double2* F, const double2* G, const double2* D, const FullMesh& fm, const Geom& g, int gap_sym);
// out = scale * mkdelta_soc(F) on the full mesh (V_Delta in Vd, Vmat host Fortran order)
void mkdelta_soc(const Geom& g, const Pairs& p, const FullMesh& fm, const double2* F, const double2* Vd,
                 const std::vector<double>& Vmat, const std::vector<int>& invschi, int gap_sym, double scale,
                 double2* out);
void initial_delta_soc(double2* D, const double* init, const double2* uni, const FullMesh& fm, const Geom& g,
                       int gap_sym);
void orb_to_band_soc(double2* out, const double2* D, const double2* uni, const FullMesh& fm, const Geom& g);

// ------------------------------------------------------- real frequency --
struct RfJob {
  double w, delta;  // real frequency and broadening of one (q, w) job
  long long qoff;   // offset of its k+q (or -k+q) index list, 0-based entries
};
// chi (or phi) matrices (Nchi, Nchi) of each job, (1/Nk) sum over the k list
void bubble_rf(double2* out, const double2* uni, const double* eig, const double* ff, const int* qsh,
               const std::vector<RfJob>& jobs, const std::vector<int>& o1, const std::vector<int>& o2, int Nk, int No,
               int Nchi, double mu, double temp, double eps, bool phi);
void rpa_trace(double2* trs, double2* tr0, const double2* chi, const double* S, const int* dmask, int Nchi, int Nq);
void trace_jobs(double2* tr, const double2* m, int Nchi, int Nq);
void pade_trace(double2* out, const double2* A, const double2* xn, const double2* wl, int Nk, int Np, int Nw, int No);
}  // namespace pgb
