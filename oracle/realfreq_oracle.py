"""CPU restatement of pyrpa's real-frequency susceptibility maps and Pade
continuation (libs/src/fchi.f90:1-318, fphi.f90:1-305, fpade.f90:1-129).

TEST INFRASTRUCTURE: this module is the checker for the GPU engine, not part
of the product.  Only tests, the smoke check and the CPU-baseline leg of the
benchmark import it.

Arrays are in the Fortran view (numpy index order equal to the Fortran one,
0-based): eig/ffermi [k, n] = eig(n, k), U [k, a, n] = uni(a, n, k); olist
holds the reference's 1-based orbital numbers.  The reference's tests do not
cover these routines, so their parity is unpinned beyond the checks in
tests/test_realfreq_oracle.py (closed forms of the Lindhard sum and exact
continuation of rational functions).
"""
from __future__ import annotations

import numpy as np

_SCALE = 1048576  # 2^20: the reference's k-coordinate key resolution


def _keys(x):
    """int(x * 2^20 + 0.5) truncated toward zero, then mod with the sign of the
    dividend, per coordinate (Fortran int and mod)."""
    i = np.trunc(x * float(_SCALE) + 0.5).astype(np.int64)
    return np.fmod(i, _SCALE)


def _lookup(klist, pts):
    keys = _keys(klist)
    table = {}
    for j, kk in enumerate(map(tuple, keys)):
        table[kk] = j                      # a repeated key keeps the last index
    out = np.zeros(len(pts), dtype=np.int64)
    for i, kk in enumerate(map(tuple, _keys(pts))):
        out[i] = table.get(kk, 0) + 1      # 1-based; a miss falls back to 1
    return out


def _wrap(t):
    t = t.copy()
    t[t >= 1.0] -= 1.0
    t[t < 0.0] += 1.0
    return t


def get_qshift(qpoint, klist):
    """1-based index of k+q on the mesh (fchi.f90:1-93)."""
    klist = np.asarray(klist, dtype=np.float64)
    return _lookup(klist, _wrap(klist + np.asarray(qpoint, dtype=np.float64)[None, :]))


def get_iqshift(qpoint, klist):
    """1-based index of -k+q on the mesh (fphi.f90:1-87)."""
    klist = np.asarray(klist, dtype=np.float64)
    return _lookup(klist, _wrap(1.0 - klist + np.asarray(qpoint, dtype=np.float64)[None, :]))


def _bubble(U, eig, ffermi, olist, qshift, weight_fn):
    """sum_k sum_lm w_klm B_i A_j / Nk with B_i = conj U(o1i, l, k+q) U(o2i, m, k),
    A_j = U(o1j, l, k+q) conj U(o2j, m, k) (fchi.f90:136-155)."""
    olist = np.asarray(olist)
    Nk = eig.shape[0]
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    kq = np.asarray(qshift) - 1
    w = weight_fn(eig[kq][:, :, None], eig[:, None, :], ffermi[kq][:, :, None], ffermi[:, None, :])  # [k, l, m]
    Ukq, Uk = U[kq], U                                          # [k, a, n]
    B = np.conj(Ukq[:, o1, :])[:, :, :, None] * Uk[:, o2, None, :]  # [k, i, l, m]
    A = Ukq[:, o1, :][:, :, :, None] * np.conj(Uk[:, o2, None, :])  # [k, j, l, m]
    return np.einsum("klm,kilm,kjlm->ij", w, B, A) / Nk


def calc_chi(U, eig, ffermi, olist, temp, qshift, w, idelta, eps):
    """fchi.f90:104-158."""
    temp_safe = max(temp, 1.0e-12)

    def weight(el, em, fl, fm):
        de = em - el
        out = np.where(np.abs(fl - fm) > eps, (fl - fm) / (w + de + 1j * idelta), 0.0)
        if abs(w) < 1.0e-12:
            out = np.where(np.abs(de) < 1.0e-9, fm * (1.0 - fm) / temp_safe + 0j, out)
        return out

    return _bubble(U, eig, ffermi, olist, qshift, weight)


def calc_phi(U, eig, ffermi, olist, mu, temp, qshift, w, idelta, eps):
    """fphi.f90:89-135."""

    def weight(el, em, fl, fm):
        den = w - em - el + 2.0 * mu
        out = -(1.0 - fl - fm) / (den + 1j * idelta)
        if idelta < eps:
            out = np.where(np.abs(den) < eps, 0.0, out)
        return out

    return _bubble(U, eig, ffermi, olist, qshift, weight)


def get_chi_irr(U, eig, ffermi, qshift, olist, wl, idelta, eps, temp):
    """chi (Nchi, Nchi, Nw) (fchi.f90:198-228)."""
    return np.stack([calc_chi(U, eig, ffermi, olist, temp, qshift, w, idelta, eps) for w in wl], axis=-1)


def get_phi_irr(U, eig, ffermi, qshift, olist, wl, idelta, eps, mu, temp):
    """phi (Nchi, Nchi, Nw) (fphi.f90:137-162)."""
    return np.stack([calc_phi(U, eig, ffermi, olist, mu, temp, qshift, w, idelta, eps) for w in wl], axis=-1)


def _diag_pairs(olist):
    olist = np.asarray(olist)
    return [l for l in range(len(olist)) if olist[l, 0] == olist[l, 1]]


def chiq_map(U, eig, ffermi, klist, S_F, olist, temp, ecut, idelta, eps, Nx, Ny):
    """(trchis, trchi) [i, j] for q = ((i)/Nx, (j)/Ny, 0) (fchi.f90:230-318):
    chi_s = (I - chi0 S)^-1 chi0, each summed over the (ll, mm) elements."""
    n = S_F.shape[0]
    d = _diag_pairs(olist)
    trs = np.zeros((Nx, Ny), dtype=np.complex128)
    tr0 = np.zeros((Nx, Ny), dtype=np.complex128)
    for i in range(Nx):
        for j in range(Ny):
            qs = get_qshift(np.array([i / Nx, j / Ny, 0.0]), klist)
            chi = calc_chi(U, eig, ffermi, olist, temp, qs, ecut, idelta, eps)
            chis = np.linalg.solve(np.eye(n) - chi @ S_F, chi)
            trs[i, j] = chis[np.ix_(d, d)].sum()
            tr0[i, j] = chi[np.ix_(d, d)].sum()
    return trs, tr0


def phiq_map(U, eig, ffermi, klist, olist, mu, temp, ecut, idelta, eps, Nx, Ny, sw_omega):
    """trphi [i, j] = trace of phi at q = (i/Nx, j/Ny, 0) (fphi.f90:234-305)."""
    wre, wim = (ecut, idelta) if sw_omega else (0.0, 0.0)
    out = np.zeros((Nx, Ny), dtype=np.complex128)
    for i in range(Nx):
        for j in range(Ny):
            qs = get_iqshift(np.array([i / Nx, j / Ny, 0.0]), klist)
            out[i, j] = np.trace(calc_phi(U, eig, ffermi, olist, mu, temp, qs, wre, wim, eps))
    return out


def get_tr_chi(chis, chi0, olist, Norb):
    """fchi.f90:160-196; chis, chi0 (Nchi, Nchi, Nw); chis_orb (Norb+2, Nw)."""
    olist = np.asarray(olist)
    Nw = chis.shape[2]
    trs = np.zeros(Nw, dtype=np.complex128)
    tr0 = np.zeros(Nw, dtype=np.complex128)
    orb = np.zeros((Norb + 2, Nw), dtype=np.complex128)
    d = _diag_pairs(olist)
    for jj in d:
        for kk in d:
            trs += chis[kk, jj]
            tr0 += chi0[kk, jj]
            if olist[jj, 0] == olist[kk, 0]:
                orb[olist[jj, 0] - 1] = chis[kk, jj]
            if olist[kk, 0] == 2 and olist[jj, 0] == 3:
                orb[Norb] = chis[kk, jj]
            if olist[kk, 0] == 2 and olist[jj, 0] == 4:
                orb[Norb + 1] = chis[kk, jj]
    return trs, tr0, orb


def get_tr_phi(phi, olist, Norb):
    """fphi.f90:164-193; phi (Nchi, Nchi, Nw); phi_orb (Norb+2, Nw)."""
    olist = np.asarray(olist)
    Nchi, Nw = phi.shape[0], phi.shape[2]
    tr = np.zeros(Nw, dtype=np.complex128)
    orb = np.zeros((Norb + 2, Nw), dtype=np.complex128)
    d = _diag_pairs(olist)
    for jj in range(Nchi):
        tr += phi[jj, jj]
        if jj in d:
            for kk in d:
                if olist[jj, 0] == olist[kk, 0]:
                    orb[olist[jj, 0] - 1] = phi[kk, jj]
                if olist[kk, 0] == 2 and olist[jj, 0] == 3:
                    orb[Norb] = phi[kk, jj]
                if olist[kk, 0] == 2 and olist[jj, 0] == 4:
                    orb[Norb + 1] = phi[kk, jj]
    return tr, orb


# --------------------------------------------------------------------------- #
#  Pade continued fraction (fpade.f90)
# --------------------------------------------------------------------------- #
def get_a(xn, data):
    """Continued-fraction coefficients a_i = g_i(z_i) (fpade.f90:1-27).  Only
    the entries j >= i of g_i enter later steps; the others are skipped here
    (the reference computes and discards them)."""
    xn = np.asarray(xn, dtype=np.complex128)
    g = np.array(data, dtype=np.complex128)
    Np = len(g)
    a = np.zeros(Np, dtype=np.complex128)
    a[0] = g[0]
    for i in range(1, Np):
        j = np.arange(i, Np)
        gj = g[j]
        den = np.where(gj == 0, 1.0 + 0j, (xn[j] - xn[i - 1]) * gj)
        new = np.where(gj == 0, 0.0 + 0j, (g[i - 1] - gj) / den)
        g[j] = new
        a[i] = g[i]
    return a


def get_QP(a, xn, wlist):
    """P_N, Q_N of the continued fraction at wlist (fpade.f90:29-55)."""
    wlist = np.asarray(wlist, dtype=np.complex128)
    P0 = np.zeros_like(wlist)
    P1 = np.full_like(wlist, a[0])
    Q0 = np.ones_like(wlist)
    Q1 = np.ones_like(wlist)
    P, Q = P1.copy(), Q1.copy()
    for i in range(1, len(a)):
        P = P1 + a[i] * (wlist - xn[i - 1]) * P0
        Q = Q1 + a[i] * (wlist - xn[i - 1]) * Q0
        P0, P1, Q0, Q1 = P1, P, Q1, Q
    return P, Q


def pade_with_trace(A, iwlist, wlist):
    """sum over orbitals of the continuation of A[k, :, o, o] (fpade.f90:77-129);
    A [k, iw, a, b] Fortran view, result [w, k] view of arrayout(Nw, Nk)."""
    Nk, Niw, No, _ = A.shape
    out = np.zeros((len(wlist), Nk), dtype=np.complex128)
    for o in range(No):
        for k in range(Nk):
            a = get_a(iwlist, A[k, :, o, o])
            P, Q = get_QP(a, iwlist, wlist)
            out[:, k] += P / Q
    return out
