/* C ABI of the GB300 FLEX / RPA / linearized-Eliashberg engine (libfmod.so).
 *
 * Each declaration replaces the Fortran bind(C) subroutine of the pyrpa
 * reference library cited beside it, with the same symbol name, argument
 * order and meaning, so pyrpa's ctypes wrappers (libs/flibs/*.py) bind it
 * unchanged.  Conventions, as in the reference:
 *   - every argument is passed by reference (scalars included);
 *   - int64_t = integer(c_int64_t), double = real(c_double),
 *     double _Complex arrays are passed as double[2*n] (re, im);
 *   - bool = logical(1) / ctypes c_bool (1 byte);
 *   - arrays are Fortran column-major: the Fortran shape is the reverse of
 *     the numpy shape the wrappers allocate, e.g. Gk(Nk,Nw,Norb,Norb) is the
 *     numpy [Norb,Norb,Nw,Nk] array;
 *   - kmap(3,Nkall) holds 0-based grid coordinates, invk(3,Nkall) the 1-based
 *     irreducible index, the 0/1 (direct / via -k) flag and the index of -k;
 *     olist(Nchi,2) the 1-based orbitals of each orbital pair.
 * Every call is synchronous.  Failures print a message, fill the outputs
 * with NaN and are reported by pyrpa_gb_last_error (the reference stops the
 * process instead).  The hot path runs on the GPU only; without a visible
 * CUDA device every entry point reports an error.
 */
#ifndef PYRPA_GB300_FMOD_H
#define PYRPA_GB300_FMOD_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ setup --- */
/* fmod.f90:7-20 openmp_params: reports no OpenMP (0, false); this library runs on the GPU */
void openmp_params(int64_t* omp_num, bool* omp_check);
/* finv.f90:1-290 generate_irr_kpoint_inv: klist(3,Nk), kmap(3,Nkall), invk(3,Nkall) */
void generate_irr_kpoint_inv(double* klist, int64_t* kmap, int64_t* invk, const int64_t* Nk,
                             const int64_t* Nx, const int64_t* Ny, const int64_t* Nz);
/* finv.f90:292-305 get_kweight */
void get_kweight(double* weight, const int64_t* invk, const int64_t* Nk, const int64_t* Nkall);
/* fmod.f90:162-207 gen_ham: ham_k(Norb,Norb,Nk) = sum_R H(R) exp(-2 pi i k.R), Hermitized */
void gen_ham(double* ham_k, const double* klist, const double* ham_r, const double* rvec,
             const int64_t* Nk, const int64_t* Nr, const int64_t* Norb);
/* fmod.f90:209-248 get_eig: eig(Norb,Nk) ascending, uni(Norb,Norb,Nk) eigenvectors in columns */
void get_eig(double* eig, double* uni, const double* ham_k, const int64_t* Nk, const int64_t* Norb);
/* fmod.f90:250-310 get_eig_mlo: eigenpairs in a non-orthogonal basis (overlap
 * Ovlk(Norb,Norb,Nk)) by canonical orthogonalization; basis directions with
 * overlap eigenvalue <= 1e-8 are dropped and leave an eigenvalue 0 */
void get_eig_mlo(double* eig, double* uni, const double* ham_k, const double* Ovlk, const int64_t* Nk,
                 const int64_t* Norb);
/* fmod.f90:312-340 get_ffermi */
void get_ffermi(double* ffermi, const double* eig, const double* mu, const double* temp,
                const int64_t* Nk, const int64_t* Norb);
/* fmod.f90:657-716 get_parity_prop: Pmn(Norb,Norb) = +-1 */
void get_parity_prop(double* Pmn, const double* rvec, const double* ham_r, const int64_t* Norb,
                     const int64_t* Nr);
/* fUJ.f90:1-57 get_scmat: Kanamori S and C (Nchi,Nchi), U' = U - 2J */
void get_scmat(double* Smat, double* Cmat, const int64_t* ol, const int64_t* site, const double* Uval,
               const double* Jval, const int64_t* Nchi);
/* fUJ.f90:59-107 get_scmat_orb: orbital-dependent Umat/Jmat (Norb,Norb) */
void get_scmat_orb(double* Smat, double* Cmat, const int64_t* ol, const int64_t* site,
                   const double* Umat, const double* Jmat, const int64_t* Nchi, const int64_t* Norb);

/* ------------------------------------------------------------ Green --- */
/* fself.f90:1-41 gen_green0 (gen_green0_): Gk(Nk,Nw,Norb,Norb) */
void gen_green0_(double* Gk, const double* eig, const double* uni, const double* mu, const double* temp,
                 const int64_t* Nk, const int64_t* Nw, const int64_t* Norb);
/* fself.f90:43-79 gen_green_inv (gen_green_inv_): Gk = iw + mu - H - Sigma */
void gen_green_inv_(double* Gk, const double* self, const double* hamk, const double* mu,
                    const double* temp, const int64_t* Nk, const int64_t* Nw, const int64_t* Norb);
/* fself.f90:134-157 getinv (getinv_): in-place inverse of each Norb x Norb block */
void getinv_(double* Gk, const int64_t* Nk, const int64_t* Nw, const int64_t* Norb);

/* ------------------------------------------------------ susceptibility --- */
/* fchi.f90:615-635 get_chi0_conv (get_chi0_conv_): irr_chi(Nchi(Nchi+1)/2,2), chi_map(Nchi,Nchi,2) int32 */
void get_chi0_conv_(double* chi, const double* Gk, const int64_t* kmap, const int64_t* invk,
                    const int32_t* irr_chi, const int32_t* chi_map, const int64_t* olist,
                    const double* temp, const int64_t* Nx, const int64_t* Ny, const int64_t* Nz,
                    const int64_t* Nw, const int64_t* Nk, const int64_t* Nkall, const int64_t* Norb,
                    const int64_t* Nchi);
/* fchi.f90:401-419 get_chi0: chi(Nk,Nw,Nchi,Nchi) by FFT convolution, plus the Stoner factor */
void get_chi0(double* chi, const double* Smat, const double* Cmat, const double* Gk,
              const int64_t* kmap, const int64_t* invk, const int64_t* olist, const double* temp,
              const int64_t* Nx, const int64_t* Ny, const int64_t* Nz, const int64_t* Nw,
              const int64_t* Nk, const int64_t* Nkall, const int64_t* Norb, const int64_t* Nchi,
              double* maxchi0s_out);
/* fchi.f90:894-918 get_chi0_tail: conv[G] - conv[G0] + analytic tau reference */
void get_chi0_tail(double* chi, const double* Smat, const double* Cmat, const double* Gk,
                   const double* eig, const double* uni, const int64_t* kmap, const int64_t* invk,
                   const int64_t* olist, const double* mu, const double* temp, const int64_t* Nx,
                   const int64_t* Ny, const int64_t* Nz, const int64_t* Nw, const int64_t* Nk,
                   const int64_t* Nkall, const int64_t* Norb, const int64_t* Nchi,
                   double* maxchi0s_out);
/* fchi.f90:319-350 get_chis: chis(Nchi,Nchi,Nw) = (I - chi0 S)^-1 chi0 */
void get_chis(double* chis, const double* chi0, const double* Smat, const int64_t* Nchi,
              const int64_t* Nw);
/* fself.f90:783-816 get_chis_chic: nu = 0 RPA spin/charge susceptibilities (Nk,Nchi,Nchi) */
void get_chis_chic(double* chis, double* chic, const double* chi, const double* Smat,
                   const double* Cmat, const int64_t* Nk, const int64_t* Nw, const int64_t* Nchi);
/* fself.f90:818-851 get_eig_or_tr_chi: max Re eigenvalue or trace on the full grid.
 * The Fortran dummy sw_eig is a default logical; the wrappers pass a 1-byte
 * c_bool, which is what this declaration reads. */
void get_eig_or_tr_chi(double* chiqout, const double* chi, const int64_t* invk,
                       const int64_t* Nkall, const int64_t* Nk, const int64_t* Nchi,
                       const bool* sw_eig);
/* fUJ.f90:318-365 get_vsigma_flex_nosoc (get_vsigma_flex_nosoc_): V_sigma in place */
void get_vsigma_flex_nosoc_(double* chi, const double* Smat, const double* Cmat, const int64_t* Nk,
                            const int64_t* Nw, const int64_t* Nchi);

/* ------------------------------------------------------------- FLEX --- */
/* fself.f90:287-781 mkself: FLEX self-consistency; sigmak(Nk,Nw,Norb,Norb), mu.
 * sw_out / sw_in write / read sigma.bin in the working directory. */
void mkself(double* sigmak, double* mu, const double* Smat, const double* Cmat, const int64_t* kmap,
            const int64_t* invk, const int64_t* olist, const double* hamk, const double* eig,
            const double* uni, const double* mu_init, const double* rfill, const double* temp,
            const int64_t* scf_loop, const double* pp, const double* eps, const int64_t* Nkall,
            const int64_t* Nk, const int64_t* Nw, const int64_t* Norb, const int64_t* Nchi,
            const int64_t* Nx, const int64_t* Ny, const int64_t* Nz, const int64_t* sub_sigma,
            const bool* sw_out, const bool* sw_in, const int64_t* m_diis, const bool* sw_rescale,
            const bool* sw_tail, const double* sigma_scale);

/* ------------------------------------------------------- Eliashberg --- */
/* feliash.f90:1-443 lin_eliash: leading eigenvalue lambda_out and gap delta(Nk,Nw,Norb,Norb);
 * chi is overwritten with the pairing vertex V_Delta as in the reference. */
void lin_eliash(double* delta, double* chi, const double* Gk, const double* uni,
                const double* init_delta, const double* Smat, const double* Cmat,
                const int64_t* olist, const double* prt, const int64_t* kmap, const int64_t* invk,
                const double* temp, const double* eps, const int64_t* Nkall, const int64_t* Nk,
                const int64_t* Nw, const int64_t* Nchi, const int64_t* Norb, const int64_t* Nx,
                const int64_t* Ny, const int64_t* Nz, const int64_t* itemax, const int64_t* gap_sym,
                const int64_t* arnoldi_m, double* lambda_out);
/* feliash.f90:445-484 mkfk_trs_nsoc (mkfk_trs_nsoc_): F = -G Delta G^dagger, Hermitized */
void mkfk_trs_nsoc_(double* fk, const double* Gk, const double* delta, const int64_t* Nk,
                    const int64_t* Nw, const int64_t* Norb);
/* feliash.f90:637-731 get_initial_delta (get_initial_delta_) */
void get_initial_delta_(double* delta, const double* init_delta, const double* uni, const int64_t* kmap,
                        const int64_t* invk, const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw,
                        const int64_t* Norb, const int64_t* gap_sym);
/* feliash.f90:787-821 remap_delta (remap_delta_): delta(Nkall,Nw,Norb,Norb) */
void remap_delta_(double* delta, const double* delta0, const double* prt, const int64_t* invk,
                  const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw, const int64_t* Norb,
                  const int64_t* gap_sym);
/* feliash.f90:733-785 conv_delta_orb_to_band: deltab(Nkall,Norb,Norb) at the first frequency */
void conv_delta_orb_to_band(double* deltab, const double* delta, const double* uni, const double* prt,
                            const int64_t* invk, const int64_t* Norb, const int64_t* Nkall,
                            const int64_t* Nk, const int64_t* Nw, const int64_t* gap_sym);

/* ------------------------------------- additions without a reference counterpart --- */
/* 64: FP64 everywhere (default, the reference's arithmetic); 32: complex FP32 FFTs,
 * contractions and vertex solves with G, Sigma, mu, DIIS and lambda kept in FP64;
 * 3264 (mixed): as 32, except that the FLEX loop of mkself / pyrpa_gb_flex_eliash
 * leaves FP32 once its residual reaches the FP32 rounding floor, continues with
 * chi0 and Sigma on FP64 bulk and the vertex on FP32, and finishes on FP64 bulk,
 * so that convergence to eps is always judged on an FP64 iteration.
 * PYRPA_GB_PRECISION=fp32 | mixed | fp64 in the environment sets it at first use. */
void pyrpa_gb_set_precision(const int64_t* bits);
void pyrpa_gb_get_precision(int64_t* bits);
/* 0 silences the progress lines the reference prints to stdout */
void pyrpa_gb_set_verbose(const int64_t* level);
/* Krylov convergence of lin_eliash (no counterpart in the reference): 0 (the
 * default) runs the reference's two passes of exactly arnoldi_m steps
 * (feliash.f90:190-388); tol > 0 restarts the pass that yields lambda from
 * its Ritz vector, arnoldi_m steps at a time (at most 12 cycles), until the
 * Ritz residual |A x - lambda x| / |lambda| = |h_{m+1,m} y_m| / |lambda| is
 * below tol.  Also PYRPA_GB_ARNOLDI_TOL. */
void pyrpa_gb_set_arnoldi_tol(const double* tol);
/* *on != 0 gives the calling host thread a context of its own: its own CUDA
 * stream, device error flags, launch counter, last error and last
 * statistics, with the process context's settings (precision, verbosity,
 * Arnoldi tolerance) copied at that moment; later settings calls from the
 * thread change only its context.  Independent problems solved from several
 * such threads overlap on the GPU (the parameter sweep packs its instances
 * this way).  *on == 0 waits for the thread's stream and hands the context
 * back for reuse.  At most 63 thread contexts exist at once.  No
 * counterpart in the reference, which runs one problem per process. */
void pyrpa_gb_set_thread_stream(const int64_t* on);
/* message of the last failure in the calling thread (NUL-terminated, at
 * most len bytes) and its code: 0 none, 1 a failure of the library or the
 * GPU, 2 an input the caller has to fix (the Python wrappers raise
 * ValueError for 2, RuntimeError for 1) */
void pyrpa_gb_last_error(char* buf, const int64_t* len, int64_t* code);
void pyrpa_gb_clear_error(void);
/* kernels launched through the calling thread's context (the process
 * context unless pyrpa_gb_set_thread_stream gave it one; all engine kernels,
 * FFT passes included) */
void pyrpa_gb_kernel_launches(int64_t* n);
/* statistics of the last mkself / lin_eliash called from this thread: iterations, esterr, Stoner, mu, lambda,
 * Eliashberg applications, then device milliseconds of chi0, vertex, Sigma, DIIS,
 * mu, Dyson, Eliashberg applications, then the FLEX iterations run on FP32 bulk,
 * the FLEX iterations of a coarse-mesh warm start and its device milliseconds,
 * the device milliseconds of the Stoner factors in the FLEX loop, and the
 * iterations of the mixed schedule's middle phase (FP64 chi0 and Sigma, FP32
 * vertex), the Ritz residual |A x - lambda x| / |lambda| of the returned
 * lambda and the Arnoldi cycles of its pass (20 doubles) */
void pyrpa_gb_last_stats(double* out);
/* real parts of the Ritz values of the last Arnoldi pass of lin_eliash /
 * lin_eliash_soc / pyrpa_gb_flex_eliash, on the operator's scale (the pass-2
 * shift undone), largest first: *count of them are kept (at most 16), the
 * first min(*n, *count) go to out.  The first is lambda.  No counterpart in
 * the reference, which prints the Ritz values (feliash.f90:309-312, 365-368). */
void pyrpa_gb_last_ritz(double* out, const int64_t* n, int64_t* count);
void pyrpa_gb_device_info(int64_t* num_sms, int64_t* device);
/* live timing of the FFT pass kernel: when on, every pass launch is bracketed
 * by CUDA events on the library stream; pyrpa_gb_fft_stats returns and resets
 * {launches, summed ms, algorithmic bytes (one read and one write per element)} */
void pyrpa_gb_fft_profile(const int64_t* on);
void pyrpa_gb_fft_stats(double* out);

/* The reference's linearized-Eliashberg driver with the FLEX self-energy
 * (libs/plibs/_calc.py:370-405: mkself -> gen_green -> get_chi0(_tail) ->
 * lin_eliash) as one call whose intermediates (G, chi0, V_Delta) stay in HBM.
 * Arguments as in mkself and lin_eliash; sigma_seed (may be NULL) replaces the
 * G0 start by a given Sigma with chemical potentials seed_mu / seed_mu_old
 * (the sw_in path without a file).  times_ms[3] (may be NULL) receives the
 * host-to-device, device compute and device-to-host milliseconds measured
 * with CUDA events on the library stream.  coarse[2] (may be NULL) = {k
 * divisor, frequency divisor}: unless both are 1 and when no sigma_seed is
 * given, the FLEX loop starts from a warm start: the model solved first on the
 * k mesh and Matsubara set divided by them (FP32 bulk, down to the FP32
 * rounding floor), its Sigma Fourier-interpolated in k to the full mesh and
 * extended in frequency with a c0 + c1/(i w) tail, its mu as the seed.  The
 * coarse H, eigenvalues and eigenvectors are taken from the fine mesh at the
 * same k.  No counterpart in the reference. */
void pyrpa_gb_flex_eliash(double* sigmak, double* mu, double* delta, double* lambda_out, double* stoner,
                          double* times_ms, const double* Smat, const double* Cmat, const int64_t* kmap,
                          const int64_t* invk, const int64_t* olist, const double* hamk, const double* eig,
                          const double* uni, const double* init_delta, const double* prt,
                          const double* sigma_seed, const double* seed_mu, const double* seed_mu_old,
                          const double* mu_init, const double* rfill, const double* temp,
                          const int64_t* scf_loop, const double* pp, const double* eps, const int64_t* Nkall,
                          const int64_t* Nk, const int64_t* Nw, const int64_t* Norb, const int64_t* Nchi,
                          const int64_t* Nx, const int64_t* Ny, const int64_t* Nz, const int64_t* sub_sigma,
                          const int64_t* m_diis, const bool* sw_rescale, const bool* sw_tail,
                          const int64_t* gap_sym, const int64_t* arnoldi_m, const int64_t* itemax,
                          const double* eps_eliash, const int64_t* coarse);

/* Nonlinear FLEX-Eliashberg loop (libs/src/ffeliash.f90:2-314, bound by
 * libs/flibs/_eliashberg.py:53-74 and called by nonlinear_eliashberg at
 * :225-300).  delta (Nk,Nw,Norb,Norb) is the seed on entry and the gap on
 * exit; Gk is the normal-state G on entry and the last self-consistent G on
 * exit; sigmak is the FLEX Sigma of the last step (zero unless sw_sigma).
 * Per iteration: Delta_new = -T/N sum V_Delta F (hermitized), convergence on
 * max|Delta_new - Delta| / max|Delta| < eps, stop once max|Delta_new| falls
 * below gap_min * max|Delta_seed|; amplitude secant on the seed shape
 * (sw_amp_newton) then DIIS over m_diis steps (linear mixing 0.3 below two
 * entries or on a singular system); optionally Sigma -> G0; then
 * G = G0 (1 + Delta F^+), F = -G0 Delta G^+ and, unless sw_Vconst, the
 * spin and charge bubbles chi_S/C = chi^GG +- chi^FF and the vertices
 * V_sigma, V_Delta.  All of it runs in FP64 on the device. */
void eliashberg(double* delta, double* sigmak, double* Gk, const double* hamk, const double* Smat,
                const double* Cmat, const int64_t* olist, const double* prt, const int64_t* kmap,
                const int64_t* invk, const double* mu, const double* temp, const double* eps,
                const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw, const int64_t* Nchi,
                const int64_t* Norb, const int64_t* Nx, const int64_t* Ny, const int64_t* Nz,
                const int64_t* itemax, const int64_t* gap_sym, const bool* sw_sigma, const bool* sw_Vconst,
                const int64_t* m_diis, const double* gap_min, const bool* sw_amp_newton);

/* Building blocks of the nonlinear loop, each one call (no counterpart symbol
 * in the reference, which keeps them internal to ffeliash.f90):
 * pyrpa_gb_chi0sc: get_chi0sc (ffeliash.f90:454-489), chi0_S = chi^GG + chi^FF
 * and chi0_C = chi^GG - chi^FF of Gk and fk (Nk,Nw,Norb,Norb) into xs, xc
 * (Nk,Nw,Nchi,Nchi); with *vertex != 0 followed by mkV_flex_nosoc
 * (ffeliash.f90:379-452): V_sigma into xs, V_Delta into xc.
 * pyrpa_gb_sc_dyson: mkgreliah_trs_nsoc then mkfkeliash_trs_nsoc
 * (ffeliash.f90:316-377): Gk = G0 (1 + delta fk^+), then fk = -G0 delta Gk^+
 * (fk in: the previous F, out: the new one). */
void pyrpa_gb_chi0sc(double* xs, double* xc, const double* Gk, const double* fk, const double* Smat,
                     const double* Cmat, const int64_t* olist, const double* prt, const int64_t* kmap,
                     const int64_t* invk, const double* temp, const int64_t* Nkall, const int64_t* Nk,
                     const int64_t* Nw, const int64_t* Nchi, const int64_t* Norb, const int64_t* Nx,
                     const int64_t* Ny, const int64_t* Nz, const int64_t* gap_sym, const int64_t* vertex);
void pyrpa_gb_sc_dyson(double* Gk, double* fk, const double* G0, const double* delta, const int64_t* Nk,
                       const int64_t* Nw, const int64_t* Norb);

/* ---- spin-orbit coupling.  Spin-orbital indices: slist(a) = +-1 spin label,
 * invs(a) = 1-based spin partner; G(-k)_ab = s_a s_b G(k)_{invs b, invs a}.
 * The engine covers Norb = 2 or 4 spin-orbitals (Nchi = 4 or 16), in FP64. */
/* fUJ.f90:109-180 / 182-251: onsite vertex V (Nchi,Nchi) from U, J or Umat, Jmat (Norb,Norb) */
void get_vmat_soc(double* Vmat, const int64_t* ol, const int64_t* sl, const int64_t* site, const int64_t* invs,
                  const double* Uval, const double* Jval, const int64_t* Nchi, const int64_t* Norb);
void get_vmat_soc_orb(double* Vmat, const int64_t* ol, const int64_t* sl, const int64_t* site,
                      const int64_t* invs, const double* Umat, const double* Jmat, const int64_t* Nchi,
                      const int64_t* Norb);
/* fselfwithsoc.f90:1-153: the FLEX loop with the spin-orbit bubble, the vertex
 * -V + V (I + chi0 V)^-1 chi0 V and the Sigma static slot -V (libs/flibs/_selfenergy.py:38-60) */
void mkself_soc(double* sigmak, double* mu, const double* Vmat, const int64_t* kmap, const int64_t* invk,
                const int64_t* invs, const int64_t* olist, const int64_t* slist, const double* hamk,
                const double* eig, const double* uni, const double* mu_init, const double* rfill,
                const double* temp, const int64_t* scf_loop, const double* pp, const double* eps,
                const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw, const int64_t* Norb,
                const int64_t* Nchi, const int64_t* Nx, const int64_t* Ny, const int64_t* Nz,
                const int64_t* sub_sigma, const bool* sw_out, const bool* sw_in, const int64_t* m_diis,
                const bool* sw_rescale, const double* sigma_scale);
/* fchi0withsoc.f90:111-214 (libs/flibs/_susceptibility.py:141-159): chi (Nk,Nw,Nchi,Nchi) plus
 * the outputs sgnsig (Norb,Norb), sgnsig2 (Nchi,Nchi) and invschi (Nchi, 1-based) */
void get_chi0_soc(double* chi, double* sgnsig, double* sgnsig2, int64_t* invschi, const double* Vmat,
                  const double* Gk, const int64_t* kmap, const int64_t* invk, const int64_t* invs,
                  const int64_t* olist, const int64_t* slist, const double* temp, const int64_t* Nx,
                  const int64_t* Ny, const int64_t* Nz, const int64_t* Nw, const int64_t* Nk,
                  const int64_t* Nkall, const int64_t* Nchi, const int64_t* Norb);
/* fchi0withsoc.f90:281-326: nu = 0 RPA channels chic, chiszz, chispm (Nk,Nchi/4,Nchi/4) */
void get_chis_chic_soc(double* chic, double* chiszz, double* chispm, const double* chi, const double* Vmat,
                       const int64_t* orb_list, const int64_t* olist, const int64_t* slist,
                       const int64_t* invs, const int64_t* Nk, const int64_t* Nw, const int64_t* Nchi,
                       const int64_t* Norb);
/* feliashwithsoc.f90:1-424: delta (Nkall,Nw,Norb,Norb) on the full mesh; chi is overwritten
 * with V_Delta = -V + V (I + chi0 V)^-1 chi0 V; two-pass Arnoldi (arnoldi_m > 0) or the
 * shifted power method.  sgnsig, sgnsig2 and prt are not read (recomputed from slist);
 * lambda goes to pyrpa_gb_last_stats. */
void lin_eliash_soc(double* delta, double* chi, const double* Gk, const double* uni,
                    const double* init_delta, const double* Vmat, const double* sgnsig, const double* sgnsig2,
                    const double* prt, const int64_t* olist, const int64_t* slist, const int64_t* kmap,
                    const int64_t* invk, const int64_t* invs, const int64_t* invschi, const double* temp,
                    const double* eps, const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw,
                    const int64_t* Nchi, const int64_t* Norb, const int64_t* Nx, const int64_t* Ny,
                    const int64_t* Nz, const int64_t* itemax, const int64_t* gap_sym, const int64_t* arnoldi_m);
/* feliashwithsoc.f90:426-518: F (Nkall,Nw,Norb,Norb) = -G(k) delta(k) G(-k)^+ and the spin-block fills */
void mkfk_trs_soc_(double* fk, const double* Gk, const double* delta, const double* sgnsig, const int64_t* slist,
                   const int64_t* invk, const int64_t* invs, const int64_t* Nkall, const int64_t* Nk,
                   const int64_t* Nw, const int64_t* Norb, const int64_t* gap_sym);
/* feliashwithsoc.f90:750-794: band-basis gap (Nkall,Norb,Norb) at the first frequency */
void conv_delta_orb_to_band_soc(double* deltab, const double* delta, const double* uni, const int64_t* invk,
                                const int64_t* invs, const int64_t* slist, const int64_t* Norb,
                                const int64_t* Nkall, const int64_t* Nk, const int64_t* Nw);

/* ---- real-frequency maps and Pade (fchi.f90:1-318, fphi.f90:1-305, fpade.f90).
 * Band data in the wrappers' layouts: uni (Norb,Norb,Nk), eig/ffermi (Norb,Nk),
 * klist (3,Nk), all on the k list the maps sum over. */
/* 1-based index of k+q (get_qshift_) / -k+q (get_iqshift_) on klist; a miss gives 1 */
void get_qshift_(const double* qpoint, const double* klist, int64_t* qshift, const int64_t* Nk);
void get_iqshift_(const double* qpoint, const double* klist, int64_t* qshift, const int64_t* Nk);
/* chi0(q, w + i idelta) (Nchi,Nchi,Nw) of the band-basis Lindhard sum at one q */
void get_chi_irr(double* chi, const double* uni, const double* eig, const double* ffermi, const int64_t* qshift,
                 const int64_t* ol, const double* wl, const int64_t* Nchi, const int64_t* Norb, const int64_t* Nk,
                 const int64_t* Nw, const double* idelta, const double* eps, const double* temp);
/* particle-particle analog phi0(q, w) (Nchi,Nchi,Nw) */
void get_phi_irr(double* phi, const double* uni, const double* eig, const double* ffermi, const int64_t* qshift,
                 const int64_t* ol, const double* wl, const int64_t* Nchi, const int64_t* Norb, const int64_t* Nk,
                 const int64_t* Nw, const double* idelta, const double* eps, const double* mu, const double* temp);
/* (ll,mm) sums of chi_s = (I - chi0 S)^-1 chi0 and chi0 at w = ecut over q = (i/Nx, j/Ny, 0);
 * trchis, trchi (Ny,Nx).  Nchi = 1, 4, 9, 16 or 25. */
void chiq_map(double* trchis, double* trchi, const double* uni, const double* eig, const double* ffermi,
              const double* klist, const double* Smat, const int64_t* ol, const double* temp, const double* ecut,
              const double* idelta, const double* eps, const int64_t* Nx, const int64_t* Ny, const int64_t* Nk,
              const int64_t* Norb, const int64_t* Nchi);
/* trace of phi over q = (i/Nx, j/Ny, 0) (trphi (Ny,Nx)); w = ecut + i idelta if *sw_omega, else 0 */
void phiq_map(double* trphi, const double* uni, const double* eig, const double* ffermi, const double* klist,
              const int64_t* ol, const double* mu, const double* temp, const double* ecut, const double* idelta,
              const double* eps, const int64_t* Nx, const int64_t* Ny, const int64_t* Nk, const int64_t* Norb,
              const int64_t* Nchi, const bool* sw_omega);
/* orbital traces per frequency (host code) */
void get_tr_chi(double* trchis, double* trchi0, double* chis_orb, const double* chis, const double* chi0,
                const int64_t* olist, const int64_t* Nw, const int64_t* Nchi, const int64_t* Norb);
void get_tr_phi(double* trphi, double* phi_orb, const double* phi, const int64_t* olist, const int64_t* Nw,
                const int64_t* Nchi, const int64_t* Norb);
/* continued-fraction coefficients and P_N, Q_N of one series (host code) */
void get_a_(double* a, const double* xn, const double* inp_data, const int64_t* Np);
void get_qp_(double* P, double* Q, const double* a, const double* xn, const double* wlist, const int64_t* Nw,
             const int64_t* Np);
/* arrayout (Nw,Nk) = sum over orbitals of the Pade continuation of arrayin(k,:,o,o) (Nk,Niw,Norb,Norb) */
void pade_with_trace(const double* arrayin, double* arrayout, const double* iwlist, const double* wlist,
                     const int64_t* Nk, const int64_t* Niw, const int64_t* Nw, const int64_t* Norb);

/* fself.f90:85-129 gen_green_inv_from_eig: G^-1 from eig(Norb,Nk) and uni(Norb,Norb,Nk):
 * Gk(Nk,Nw,Norb,Norb) = sum_n uni(m,n,k) conj(uni(l,n,k)) (iw + mu - eig(n,k)) - self */
void gen_green_inv_from_eig(double* Gk, const double* self, const double* uni, const double* eig, const double* mu,
                            const double* temp, const int64_t* Nk, const int64_t* Nw, const int64_t* Norb);

/* Symbols outside the accelerated path (transport, impurity, Eilenberger ...) are exported with no
 * arguments read and report "not part of the GB300 FLEX/RPA/Eliashberg engine"
 * so that `import libs.flibs` binds every name it expects. */

/* plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182) without the file I/O:
 * sigma (Nk,Nw_old,Norb,Norb) of the Matsubara mesh at temp_old onto Nw_new
 * frequencies at temp_new (evaluated at w_scale * w_n(temp_new)): cubic
 * spline over the conjugate-extended axis, c0 + c1/(iw) tail beyond the kept
 * cutoff, diagonal clipped to Im <= 0.  The reference does this in Python;
 * pyrpa_gb300.seed.regrid_sigma_bin wraps it with the sigma.bin I/O. */
void pyrpa_gb_regrid_sigma(double* out, const double* sigma, const int64_t* Nk, const int64_t* Nw_old,
                           const int64_t* Nw_new, const int64_t* Norb, const double* temp_old,
                           const double* temp_new, const double* w_scale);

/* plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182) with its file handling:
 * reads the io_sigma records of in_path (fself.f90:742-780), checks temp_old,
 * Norb and Nw_old against the (temp, Nw, Norb, Nk) record when the file has
 * one (NaN / 0 = take the file's value; Nw_new 0 = keep Nw_old), regrids as
 * pyrpa_gb_regrid_sigma and writes mu, mu_OLD, the new Sigma and the record
 * of the new mesh to out_path.  *Nk_out, *Nw_new_out = the written shape, or
 * -1 with pyrpa_gb_last_error code 2 when the file or an argument is at fault. */
void pyrpa_gb_regrid_sigma_file(const char* in_path, const char* out_path, const double* temp_old,
                                const double* temp_new, const int64_t* Norb, const int64_t* Nw_old,
                                const int64_t* Nw_new, const double* w_scale, int64_t* Nk_out,
                                int64_t* Nw_new_out);

/* The k -> R step of plibs.output_self_wannier / output_gap_wannier
 * (libs/plibs/_wannier_io.py:52-98): data in the wrappers' layout
 * [Norb][Norb][Nw][Nk_data] (Nk_data = irreducible count, complex conjugate at
 * -k; or Nkall, full grid) -> inverse FFT over the k mesh (1/Nkall) of the
 * first min(Ncut, Nw) frequencies, out [Norb][Norb][Ncut][Nz][Ny][Nx].
 * pyrpa_gb300.wannier does the zeroing, R selection and file output. */
void pyrpa_gb_wannier_r(double* out, const double* data, const int64_t* kmap, const int64_t* invk,
                        const int64_t* Nx, const int64_t* Ny, const int64_t* Nz, const int64_t* Nk_data,
                        const int64_t* Nw, const int64_t* Norb, const int64_t* Ncut);

/* ------------------------------------------------------ FFT tuning --- */
/* No counterpart in the reference.  The settings the FFT autotuner
 * (PYRPA_GB_FFT_TUNE=1) may try for one axis of length n with elem_bytes-byte
 * elements: out[2i] = L1 (four-step split, 0 = one pass or the heuristic),
 * out[2i+1] = lines per CTA (0 = the heuristic), the heuristic first; at most
 * cap pairs are written, count = all of them.  Host only: needs no GPU. */
void pyrpa_gb_fft_candidates(const int64_t* n, const int64_t* elem_bytes, int64_t* out, const int64_t* cap,
                             int64_t* count);

/* ------------------------------------------------ coarse-mesh seed --- */
/* No counterpart in the reference (a pyrpa user seeds mkself by hand through
 * sigma.bin, fself.f90:742-780).  sig_c (Nk_c,Nw_c,Norb,Norb) on the coarse
 * irreducible mesh (kmap_c, invk_c) -> sig_f (Nk_f,Nw_f,Norb,Norb) on the fine
 * one: Fourier interpolation over k (each coarse axis divides the fine one;
 * an even axis's Nyquist plane is split in half), and for n >= Nw_c the
 * c0 + c1/(i w) tail through the coarse frequencies 3 Nw_c / 4 and Nw_c - 2
 * (0-based), as plibs.regrid_sigma_bin (libs/plibs/_calc.py:52-182) extends
 * its tail.  Norb <= 8. */
void pyrpa_gb_sigma_interp(double* sig_f, const double* sig_c, const int64_t* kmap_c, const int64_t* invk_c,
                           const int64_t* Nx_c, const int64_t* Ny_c, const int64_t* Nz_c, const int64_t* Nk_c,
                           const int64_t* Nw_c, const int64_t* kmap_f, const int64_t* invk_f, const int64_t* Nx_f,
                           const int64_t* Ny_f, const int64_t* Nz_f, const int64_t* Nk_f, const int64_t* Nw_f,
                           const int64_t* Norb, const double* temp);

/* ----------------------------------------------- learned warm start --- */
/* No counterpart in the reference.  A network refines the interpolated seed
 * Sigma before the fine FLEX loop.  One row per (k, n, band i, band j) of the
 * fine mesh: 16 features of U^dagger Sigma_seed U, the band energies, w_n and
 * the model's descriptors desc[9] = {U, J, T, fill, Stoner factor of the
 * coarse solve, mu of the coarse solve, band width W, max |Sigma_seed|,
 * Norb} -> 16 -> 64 -> 64 -> 2 (tanh) -> the band-basis correction in units
 * of max |Sigma_seed|.  FP32 weights (5378, flat: W1[64][16], b1, W2[64][64],
 * b2, W3[2][64], b3), bf16 inputs and activations, FP32 gradients, Adam.
 * A handle names one network with its training rows in HBM.  Arrays in the
 * layouts above: sigma (Nk,Nw,Norb,Norb), uni (Norb,Norb,Nk), eig (Norb,Nk);
 * kn [npairs][2] = (k, n) 0-based.  Norb <= 8. */
void pyrpa_gb_lws_create(int64_t* handle);
void pyrpa_gb_lws_destroy(const int64_t* handle);
/* theta[n], n = 5378; setting the parameters resets the Adam state */
void pyrpa_gb_lws_set_params(const int64_t* handle, const float* theta, const int64_t* n);
void pyrpa_gb_lws_get_params(const int64_t* handle, float* theta, const int64_t* n);
/* appends npairs * Norb^2 rows (features of sig_seed, targets sig_fine - sig_seed) */
void pyrpa_gb_lws_add_samples(const int64_t* handle, const double* sig_seed, const double* sig_fine,
                              const double* uni, const double* eig, const int64_t* kn, const int64_t* npairs,
                              const int64_t* Nk, const int64_t* Nw, const int64_t* Nw_c, const int64_t* Norb,
                              const double* desc);
void pyrpa_gb_lws_clear_samples(const int64_t* handle);
void pyrpa_gb_lws_num_samples(const int64_t* handle, int64_t* rows);
/* x [rows][16] (the bf16 features as float), t [rows][2] when sig_fine is not NULL */
void pyrpa_gb_lws_features(float* x, float* t, const double* sig_seed, const double* sig_fine, const double* uni,
                           const double* eig, const int64_t* kn, const int64_t* npairs, const int64_t* Nk,
                           const int64_t* Nw, const int64_t* Nw_c, const int64_t* Norb, const double* desc);
/* y [rows][2] of x [rows][16] */
void pyrpa_gb_lws_forward(const int64_t* handle, const float* x, const int64_t* rows, float* y);
/* mean over the training rows of sum (y - t)^2, and its gradient grad[5378] */
void pyrpa_gb_lws_loss_grad(const int64_t* handle, double* loss, float* grad);
/* one Adam step with the whole training set's gradient; loss before the step */
void pyrpa_gb_lws_step(const int64_t* handle, const double* lr, const double* beta1, const double* beta2,
                       const double* eps, double* loss);
/* steps Adam steps on batches drawn uniformly with replacement (mt19937_64(seed)); loss[steps] */
void pyrpa_gb_lws_train(const int64_t* handle, const int64_t* steps, const int64_t* batch, const double* lr,
                        const double* beta1, const double* beta2, const double* eps, const int64_t* seed,
                        double* loss);
/* sigma (in place) += U (max|sigma| * y) U^dagger at every (k, n) */
void pyrpa_gb_lws_apply(const int64_t* handle, double* sigma, const double* uni, const double* eig,
                        const int64_t* Nk, const int64_t* Nw, const int64_t* Nw_c, const int64_t* Norb,
                        const double* desc);

/* Allocation-free variant of get_eig_or_tr_chi.  No counterpart in the reference.
 * All pointers are DEVICE pointers in the layouts of get_eig_or_tr_chi: chi
 * (Nk,Nchi,Nchi) complex128, invk (3,Nkall) int64, chiqout (Nkall) complex128.
 * The work is enqueued on `stream` (a cudaStream_t; NULL = the default stream)
 * and the call returns without waiting; chiqout is ready when the stream gets
 * there.  It allocates no device memory: the per-q scratch is a fixed 1 MiB
 * device array, so Nk is limited to 65,536 (larger Nk is rejected with an
 * error).  Nothing in the scratch has to start at zero: each call writes the
 * Nk values it reads.  An invk(1,i) outside [1,Nk] gives NaN at chiqout(i).
 * The first call on a device does a one-time set-up: it looks up the
 * scratch address and launches each kernel once, empty.  Under CUDA's lazy
 * module loading (the default) that is when the library's module and the
 * eigenvalue kernel's per-thread local memory are mapped on the device, so
 * make that first call before the host's allocator reserves most of HBM, and
 * before any stream capture; later calls take no device memory.  Calls whose work overlaps on
 * the device (different streams, or threads) share the one scratch array and
 * race: order them on one stream.  Returns 0 on success, 1 on an error whose
 * message pyrpa_gb_last_error returns. */
int pyrpa_gb_eig_or_tr_chi_noalloc(void* chiqout, const void* chi, const int64_t* invk, int64_t Nkall,
                                   int64_t Nk, int64_t Nchi, int32_t sw_eig, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PYRPA_GB300_FMOD_H */
