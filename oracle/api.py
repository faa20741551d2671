"""flibs-shaped facade over the FP64 oracle (test infrastructure only).

Same function names, argument order and Python array layouts as the pyrpa
ctypes wrappers (``libs/flibs/*.py``), so a parity test can call the oracle
and the CUDA library through identical calls.  Conversions: a Python array
of shape [A,B,...] is the Fortran array of shape (...,B,A); the oracle works
on the Fortran view (``x.T`` for the 4-D tensors).
"""
from __future__ import annotations

import numpy as np

from . import flex_oracle as O


def gen_irr_k_TRS(Nx, Ny, Nz):
    return O.generate_irr_kpoint_inv(Nx, Ny, Nz)


def gen_kpoint_weight(invk, Nk):
    return O.get_kweight(np.asarray(invk), Nk)


def gen_ham(klist, ham_r, rvec):
    return np.ascontiguousarray(O.gen_ham_F(klist, ham_r, rvec).transpose(0, 2, 1))


def get_eig(hamk):
    w, v = O.get_eig_F(hamk.transpose(0, 2, 1))
    return w, np.ascontiguousarray(v.transpose(0, 2, 1))


def get_eig_mlo(hamk, Ovlk):
    w, v = O.get_eig_mlo_F(hamk.transpose(0, 2, 1), Ovlk.transpose(0, 2, 1))
    return w, np.ascontiguousarray(v.transpose(0, 2, 1))


def get_ffermi(eig, mu, temp):
    return O.get_ffermi(eig, mu, temp)


def gen_SCmatrix(olist, site, U, J):
    return O.get_scmat(np.asarray(olist), np.asarray(site), U, J)


def gen_SCmatrix_orb(olist, site, Umat, Jmat):
    return O.get_scmat_orb(np.asarray(olist), np.asarray(site), Umat, Jmat)


def get_chi_orb_list(Norb, site_prof=(1,)):
    return O.get_chi_orb_list(Norb, site_prof)


def gen_Green0(eig, uni, mu, temp, Nw):
    return np.ascontiguousarray(O.gen_green0_F(eig, uni.transpose(0, 2, 1), mu, temp, Nw).T)


def gen_green(selfen, hamk, mu, temp):
    return np.ascontiguousarray(O.gen_green_F(selfen.T, hamk.transpose(0, 2, 1), mu, temp).T)


def gen_green_inv_from_eig(selfen, eig, uni, mu, temp):
    return np.ascontiguousarray(O.gen_green_inv_from_eig_F(selfen.T, eig, uni.transpose(0, 2, 1), mu, temp).T)


def _grid(kmap, invk, Nx, Ny, Nz):
    return O.KGrid(np.asarray(kmap), np.asarray(invk), Nx, Ny, Nz)


def get_chi0_conv(Gk, kmap, invk, olist, temp, Nx, Ny, Nz):
    chi = O.get_chi0_conv(Gk.T, _grid(kmap, invk, Nx, Ny, Nz), np.asarray(olist), temp)
    return np.ascontiguousarray(chi.T)


def get_chi0(Smat, Cmat, Gk, olist, kmap, invk, temp, Nx, Ny, Nz):
    chi = O.get_chi0_conv(Gk.T, _grid(kmap, invk, Nx, Ny, Nz), np.asarray(olist), temp)
    st = O.ckchi(chi, Smat.T, Cmat.T)[0]
    return np.ascontiguousarray(chi.T), st


def get_chi0_tail(Smat, Cmat, Gk, eig, uni, olist, kmap, invk, mu, temp, Nx, Ny, Nz):
    chi = O.chi0_tail(Gk.T, eig, uni.transpose(0, 2, 1), mu, _grid(kmap, invk, Nx, Ny, Nz),
                      np.asarray(olist), temp)
    st = O.ckchi(chi, Smat.T, Cmat.T)[0]
    return np.ascontiguousarray(chi.T), st


def get_chis(chi0, Smat):
    X = chi0.transpose(0, 2, 1)
    return np.ascontiguousarray(O.get_chis_F(X, Smat.T).transpose(0, 2, 1))


def get_chis_chic(chi, Smat, Cmat):
    s, c = O.get_chis_chic_F(chi.T, Smat.T, Cmat.T)
    return np.ascontiguousarray(s.T), np.ascontiguousarray(c.T)


def get_eig_or_tr_chi(chi, invk, sw_eig):
    return O.get_eig_or_tr_chi(chi.T, np.asarray(invk), sw_eig)


def _fortran_view(a, shape):
    """Memory of a C-contiguous array read as a Fortran array of ``shape``."""
    return np.ascontiguousarray(a).reshape(-1).reshape(shape, order="F")


def get_Vsigma_nosoc_flex(chi, Smat, Cmat):
    """The reference wrapper passes Nk=len(chi), Nw=len(chi[0]) and lets the
    library read the buffer as (Nk,Nw,Nchi,Nchi) (libs/flibs/_selfenergy.py:60-73)."""
    Nk, Nw, Nchi = len(chi), len(chi[0]), len(Smat)
    flat = np.ascontiguousarray(chi).reshape(-1).copy()
    n = Nk * Nw * Nchi * Nchi
    if n > flat.size:
        raise ValueError("chi is smaller than the Nk*Nw*Nchi^2 elements the wrapper makes the library read")
    X = flat[:n].reshape((Nk, Nw, Nchi, Nchi), order="F")
    flat[:n] = O.vsigma_flex_nosoc(X, Smat.T, Cmat.T).reshape(-1, order="F")
    return flat.reshape(chi.shape)


def mkself(Smat, Cmat, kmap, invk, olist, hamk, eig, uni, mu, fill, temp, Nw, Nx, Ny, Nz,
           sw_out=False, sw_in=False, sub_sigma=1, scf_loop=300, eps=1.0e-4, pp=0.3, m_diis=5,
           sw_rescale=False, sw_tail=False, sigma_scale=1.0, full=False):
    r = O.mkself(Smat.T, Cmat.T, np.asarray(kmap), np.asarray(invk), np.asarray(olist),
                 hamk.transpose(0, 2, 1), eig, uni.transpose(0, 2, 1), mu, fill, temp, scf_loop,
                 pp, eps, Nx, Ny, Nz, Nw, sub_sigma=sub_sigma, m_diis=m_diis,
                 sw_rescale=sw_rescale, sw_tail=sw_tail)
    sig = np.ascontiguousarray(r.sigma.T)
    return (sig, r.mu, r) if full else (sig, r.mu)


def linearized_eliashberg(chi, Gk, uni, init_delta, Smat, Cmat, olist, plist, kmap, invk,
                          Nx, Ny, Nz, temp, gap_sym, eps=1.0e-5, itemax=300, arnoldi_m=10,
                          full=False, arnoldi_tol=0.0):
    r = O.lin_eliash(chi.T, Gk.T, uni.transpose(0, 2, 1), np.asarray(init_delta).T,
                     Smat.T, Cmat.T, np.asarray(olist), np.asarray(plist), np.asarray(kmap),
                     np.asarray(invk), temp, eps, Nx, Ny, Nz, itemax, gap_sym, arnoldi_m,
                     arnoldi_tol=arnoldi_tol)
    gap = np.ascontiguousarray(r.delta.T)
    return (gap, r.lam, r) if full else (gap, r.lam)


def get_initial_gap(klist, Norb, gap_sym):
    """Band-basis initial gap [Norb, Nk] (libs/plibs/_response.py:415-462,
    gap_symms): p+ip (gap_sym -3) is complex."""
    A = 2 * np.pi
    kx, ky, kz = klist[:, 0], klist[:, 1], klist[:, 2]
    rows = {0: np.ones(len(klist)), 1: np.cos(A * kx) - np.cos(A * ky),
            2: 2 * np.cos(A * kx) * np.cos(A * ky), 3: 2 * np.sin(A * kx) * np.sin(A * ky),
            4: 2 * np.sin(A * kx) * np.sin(A * kz), 5: 2 * np.sin(A * ky) * np.sin(A * kz),
            -1: 2 * np.sin(A * kx), -2: 2 * np.sin(A * ky), -3: 2 * np.sin(A * kx) + 2j * np.sin(A * ky)}
    row = rows.get(gap_sym, np.zeros(len(klist)))
    return np.tile(row, (Norb, 1))


def mkfk_trs_nsoc(Gk, delta):
    return np.ascontiguousarray(O.mkfk_F(Gk.T, delta.T).T)


def get_initial_delta(init_delta, uni, invk, Nw, gap_sym):
    d = O.get_initial_delta(np.asarray(init_delta).T, uni.transpose(0, 2, 1), np.asarray(invk),
                            Nw, gap_sym)
    return np.ascontiguousarray(d.T)


def conv_delta_orb_to_band(delta, uni, invk, plist, gap_sym):
    out = O.conv_delta_orb_to_band_F(delta.T, uni.transpose(0, 2, 1), np.asarray(plist),
                                     np.asarray(invk), gap_sym)
    return np.ascontiguousarray(out.T)


def get_plist(rvec, ham_r):
    P = O.get_parity_prop(rvec, ham_r)
    return np.sign(P.T[0, :])


def get_chi0sc(Gk, Fk, Smat, Cmat, olist, plist, kmap, invk, Nx, Ny, Nz, temp, gap_sym, vertex=False):
    """chi0_S, chi0_C (ffeliash.f90:454-489) or V_sigma, V_Delta (379-452), wrapper layout."""
    grid = _grid(kmap, invk, Nx, Ny, Nz)
    singlet = gap_sym >= 0
    xs, xc = O.get_chi0sc(Gk.T, Fk.T, grid, np.asarray(olist), np.asarray(plist, dtype=np.float64), temp, singlet)
    if vertex:
        xs, xc = O.mkV_flex_sc(xs, xc, Smat.T, Cmat.T, singlet)
    return np.ascontiguousarray(xs.T), np.ascontiguousarray(xc.T)


def sc_dyson(G0, Fk, delta):
    """G = G0 (1 + delta Fk^+), F = -G0 delta G^+ (ffeliash.f90:316-377)."""
    G = O.mkgreliah_F(G0.T, Fk.T, delta.T)
    F = O.mkfkeliash_F(G0.T, G, delta.T)
    return np.ascontiguousarray(G.T), np.ascontiguousarray(F.T)


def nonlinear_eliashberg(delta_init, Gk, hamk, Smat, Cmat, olist, plist, kmap, invk, mu, temp, gap_sym, Nx, Ny, Nz,
                         sw_sigma=False, sw_Vconst=False, eps=1.0e-4, itemax=100, m_diis=5, gap_min=1.0e-2,
                         sw_amp_newton=True, full=False):
    """libs/flibs/_eliashberg.py nonlinear_eliashberg; like the library, Gk is
    overwritten with the final G."""
    Nk = delta_init.shape[-1]
    sig0 = np.zeros_like(delta_init)
    r = O.nonlinear_eliashberg(np.asarray(delta_init).T, sig0.T, Gk.T, hamk.transpose(0, 2, 1), Smat.T, Cmat.T,
                               np.asarray(olist), np.asarray(plist, dtype=np.float64), np.asarray(kmap),
                               np.asarray(invk), mu, temp, eps, Nx, Ny, Nz, itemax, gap_sym, sw_sigma, sw_Vconst,
                               m_diis, gap_min, sw_amp_newton)
    Gk[...] = r.G.T
    delta, sigma = np.ascontiguousarray(r.delta.T), np.ascontiguousarray(r.sigma.T)
    return (delta, sigma, r) if full else (delta, sigma)


# ----------------------------------------------------------------- spin-orbit
# Facades of the reference's spin-orbit wrappers (libs/flibs/_interaction.py:
# gen_Vmatrix(_orb), _susceptibility.py: get_chi0_soc, get_chis_chic_soc,
# _selfenergy.py: mkself_soc, _eliashberg.py: linearized_eliashberg_soc,
# conv_delta_orb_to_band_soc, gen_Fk_soc), in the wrappers' array layouts.
from . import soc_oracle as SO  # noqa: E402


def gen_Vmatrix(olist, slist, site, invs, U, J):
    return np.ascontiguousarray(SO.get_vmat_soc(np.asarray(olist), slist, np.asarray(site), invs, U, J).T)


def gen_Vmatrix_orb(olist, slist, site, invs, Umat, Jmat):
    V = SO.get_vmat_soc(np.asarray(olist), slist, np.asarray(site), invs, 0.0, 0.0, Umat=np.asarray(Umat).T,
                        Jmat=np.asarray(Jmat).T)
    return np.ascontiguousarray(V.T)


def get_chi0_soc(Vmat, Gk, olist, slist, kmap, invk, invs, temp, Nx, Ny, Nz, full=False):
    grid = _grid(kmap, invk, Nx, Ny, Nz)
    ol = np.asarray(olist)
    chi = SO.get_chi0_conv_soc(Gk.T, grid, ol, invs, slist, temp)
    sg, sg2 = SO.sign_tables(ol, slist)
    invschi = SO.get_invschi(ol, invs)
    out = (np.ascontiguousarray(chi.T), np.ascontiguousarray(sg.T), np.ascontiguousarray(sg2.T), invschi)
    return out + (SO.ckchi_soc(chi, np.asarray(Vmat).T),) if full else out


def soc_orb_list(olist, slist, invs):
    """orb_list of get_chis_chic_soc (libs/flibs/_susceptibility.py:544-555)."""
    olist = np.asarray(olist)
    slist = np.asarray(slist)
    invs = np.asarray(invs)
    orbs = np.where(slist == 1)[0]
    o1, o2 = np.meshgrid(orbs, orbs)
    pairs = np.array([o1.flatten(), o2.flatten()]).T
    out = np.zeros(len(olist), dtype=np.int64)
    for i, ol in enumerate(olist):
        a = (ol[0] if slist[ol[0] - 1] == 1 else invs[ol[0] - 1]) - 1
        b = (ol[1] if slist[ol[1] - 1] == 1 else invs[ol[1] - 1]) - 1
        for j, pb in enumerate(pairs):
            if a == pb[0] and b == pb[1]:
                out[i] = j + 1
                break
    return out


def get_chis_chic_soc(chi, Vmat, olist, slist, invs):
    ol = np.asarray(olist)
    orb_list = soc_orb_list(ol, slist, invs)
    c, sz, pm = SO.get_chis_chic_soc(chi.T, np.asarray(Vmat).T, orb_list, ol, slist)
    return np.ascontiguousarray(c.T), np.ascontiguousarray(sz.T), np.ascontiguousarray(pm.T)


def mkself_soc(Vmat, kmap, invk, invs, olist, slist, hamk, eig, uni, mu, fill, temp, Nw, Nx, Ny, Nz,
               sw_out=False, sw_in=False, sub_sigma=1, scf_loop=300, eps=1.0e-4, pp=0.3, m_diis=5,
               sw_rescale=False, sigma_scale=1.0, full=False):
    r = SO.mkself_soc(np.asarray(Vmat).T, np.asarray(kmap), np.asarray(invk), invs, np.asarray(olist), slist,
                      hamk.transpose(0, 2, 1), eig, uni.transpose(0, 2, 1), mu, fill, temp, scf_loop, pp, eps,
                      Nx, Ny, Nz, Nw, sub_sigma=sub_sigma, m_diis=m_diis, sw_rescale=sw_rescale)
    sig = np.ascontiguousarray(r.sigma.T)
    return (sig, r.mu, r) if full else (sig, r.mu)


def linearized_eliashberg_soc(chi, Gk, uni, init_delta, Vmat, sgnsig, sgnsig2, plist, slist, olist, kmap, invk,
                              invs, invschi, Nx, Ny, Nz, temp, gap_sym, eps=1.0e-4, itemax=300, arnoldi_m=10,
                              full=False):
    """Like the library, chi is overwritten with the pairing vertex."""
    r, Vd = SO.lin_eliash_soc(chi.T, Gk.T, uni.transpose(0, 2, 1), np.asarray(init_delta).T, np.asarray(Vmat).T,
                              np.asarray(olist), slist, np.asarray(kmap), np.asarray(invk), invs, temp, eps, Nx, Ny,
                              Nz, itemax, gap_sym, arnoldi_m)
    chi[...] = Vd.T
    gap = np.ascontiguousarray(r.delta.T)
    return (gap, r.lam, r) if full else gap


def conv_delta_orb_to_band_soc(delta, uni, invk, invs, slist):
    out = SO.conv_delta_orb_to_band_soc(delta.T, uni.transpose(0, 2, 1), np.asarray(invk), invs, slist)
    return np.ascontiguousarray(out.T)


def gen_Fk_soc(Gk, delta, invk, invs, slist, gap_sym):
    F = SO.mkfk_trs_soc(Gk.T, delta.T, slist, np.asarray(invk), invs, gap_sym)
    return np.ascontiguousarray(F.T)


# ------------------------------------------------------- real-frequency maps
# Facades of libs/flibs/_susceptibility.py (get_chi_irr, chis_qmap, get_tr_chi,
# get_phi_irr, phi_qmap, get_tr_phi), _hamiltonian.py (get_qshift,
# get_iqshift) and _green.py (get_a, get_QP, pade_with_trace), wrapper layouts.
from . import realfreq_oracle as RF  # noqa: E402


def get_qshift(klist, qpoint):
    return RF.get_qshift(qpoint, klist)


def get_iqshift(klist, qpoint):
    return RF.get_iqshift(qpoint, klist)


def get_chi_irr(uni, eig, ffermi, qshift, olist, wlist, idelta, temp):
    chi = RF.get_chi_irr(uni.transpose(0, 2, 1), eig, ffermi, qshift, np.asarray(olist), np.asarray(wlist),
                         idelta, idelta * 1e-3, temp)
    return np.ascontiguousarray(chi.T)


def chis_qmap(uni, eig, ffermi, klist, Smat, olist, Nx, Ny, temp, ecut, idelta):
    return RF.chiq_map(uni.transpose(0, 2, 1), eig, ffermi, np.asarray(klist), np.asarray(Smat).T,
                       np.asarray(olist), temp, ecut, idelta, idelta * 1e-3, Nx, Ny)


def get_tr_chi(chis, chi0, olist):
    ol = np.asarray(olist)
    trs, tr0, orb = RF.get_tr_chi(chis.T, chi0.T, ol, int(ol.max()))
    return trs, tr0, np.ascontiguousarray(orb.T)


def get_phi_irr(uni, eig, ffermi, qshift, olist, wlist, idelta, mu, temp):
    phi = RF.get_phi_irr(uni.transpose(0, 2, 1), eig, ffermi, qshift, np.asarray(olist), np.asarray(wlist),
                         idelta, idelta * 1e-3, mu, temp)
    return np.ascontiguousarray(phi.T)


def phi_qmap(uni, eig, ffermi, klist, olist, Nx, Ny, mu, temp, ecut, idelta, sw_omega):
    return RF.phiq_map(uni.transpose(0, 2, 1), eig, ffermi, np.asarray(klist), np.asarray(olist), mu, temp, ecut,
                       idelta, idelta * 1e-3, Nx, Ny, sw_omega)


def get_tr_phi(phi, olist):
    ol = np.asarray(olist)
    tr, orb = RF.get_tr_phi(phi.T, ol, int(ol.max()))
    return tr, np.ascontiguousarray(orb.T)


def get_a(inp_data, xlist):
    return RF.get_a(xlist, inp_data)


def get_QP(a, xlist, wlist):
    P, Q = RF.get_QP(a, xlist, wlist)
    return Q, P  # the reference wrapper returns (Q, P)


def pade_with_trace(A, iwlist, wlist):
    return np.ascontiguousarray(RF.pade_with_trace(A.T, iwlist, wlist).T)
