"""CPU restatement of the spin-orbit-coupled FLEX / linearized-Eliashberg
path of pyrpa (libs/src/fchi0withsoc.f90, fselfwithsoc.f90,
feliashwithsoc.f90, fUJ.f90:109-251,367-399).

TEST INFRASTRUCTURE: this module is the checker for the GPU engine, not part
of the product.  Only tests, the smoke check and the CPU-baseline leg of the
benchmark import it.

Conventions as in flex_oracle: "Fortran view" arrays (numpy index order equal
to the Fortran one, 0-based); olist holds the reference's 1-based orbital
numbers; invs is the reference's 1-based spin-partner list and slist its +-1
spin labels.  Orbital indices inside the functions are 0-based.

Parity of this restatement is unpinned: the reference's test suite has no
case for the spin-orbit path, so it is checked only against the GPU engine
and against its own limits (see tests/test_soc_oracle.py).
"""
from __future__ import annotations

import numpy as np

from .flex_oracle import (KGrid, _reverse_all, _zgeev_vector, chi0_threshold, gen_green0_F, gen_green_F,
                          hf_subtract, matsubara, mkself, pad_boson)


# --------------------------------------------------------------------------- #
#  interaction and index tables
# --------------------------------------------------------------------------- #
def get_vmat_soc(olist, slist, site, invs, U, J, Umat=None, Jmat=None):
    """Onsite vertex with spin-orbit coupling, V[j,i] in the Fortran view
    (fUJ.f90:109-180; with Umat/Jmat the orbital-dependent form of :182-251).
    The branch structure of the reference is kept case by case."""
    olist = np.asarray(olist)
    Nchi = len(olist)
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    s = np.asarray(slist)
    inv = np.asarray(invs) - 1
    V = np.zeros((Nchi, Nchi))
    orb = Umat is not None
    Up = U - 2 * J
    for i in range(Nchi):
        for j in range(Nchi):
            if site[i] != site[j]:
                continue
            if s[o1[i]] == s[o2[i]] and s[o1[j]] == s[o2[j]]:
                if s[o1[i]] == s[o1[j]]:                       # same-spin density: (C-S)/2
                    if o1[i] == o2[j] and o1[j] == o2[i]:
                        continue
                    if o1[i] == o2[i] and o1[j] == o2[j]:
                        V[j, i] = (Umat[o1[i], o1[j]] - Jmat[o1[i], o1[j]]) if orb else Up - J
                    elif o1[i] == o1[j] and o2[i] == o2[j]:
                        V[j, i] = (Jmat[o1[i], o2[i]] - Umat[o1[i], o2[i]]) if orb else J - Up
                else:                                           # opposite-spin density: (C+S)/2
                    if o1[i] == o2[i] and o1[j] == o2[j]:
                        if o1[i] == inv[o1[j]]:
                            V[j, i] = Umat[o1[i], o1[i]] if orb else U
                        else:
                            V[j, i] = Umat[o1[i], o1[j]] if orb else Up
                    elif o1[i] == inv[o1[j]] and o2[i] == inv[o2[j]]:
                        V[j, i] = Jmat[o1[i], o2[i]] if orb else J
                    elif o1[i] == inv[o2[j]] and o1[j] == inv[o2[i]]:
                        V[j, i] = Jmat[o1[i], o2[i]] if orb else J
            elif s[o1[i]] == s[o1[j]] and s[o2[i]] == s[o2[j]]:  # spin flip: -S
                if o1[i] == inv[o2[i]] and o1[j] == inv[o2[j]]:
                    if o1[i] == o1[j]:
                        V[j, i] = -(Umat[o1[i], o1[i]] if orb else U)
                    else:
                        V[j, i] = -(Jmat[o1[i], o1[j]] if orb else J)
                elif o1[i] == o1[j] and o2[i] == o2[j]:
                    V[j, i] = -(Umat[o1[i], o2[i]] if orb else Up)
                elif o1[i] == inv[o2[j]] and o1[j] == inv[o2[i]]:
                    V[j, i] = -(Jmat[o1[i], o2[i]] if orb else J)
    return V


def sign_tables(olist, slist):
    """sgnsig[i,j] = s_i s_j and sgnsig2[l,m] = s_l1 s_l2 s_m1 s_m2
    (fchi0withsoc.f90:136-154)."""
    olist = np.asarray(olist)
    s = np.asarray(slist, dtype=np.float64)
    sgnsig = np.outer(s, s)
    p = s[olist[:, 0] - 1] * s[olist[:, 1] - 1]
    return sgnsig, np.outer(p, p)


def get_invschi(olist, invs):
    """1-based chi index of the spin-flipped pair, 0 where none (fchi0withsoc.f90:200-214)."""
    olist = np.asarray(olist)
    inv = np.asarray(invs)
    Nchi = len(olist)
    out = np.zeros(Nchi, dtype=np.int64)
    for l in range(Nchi):
        i, j = inv[olist[l, 0] - 1], inv[olist[l, 1] - 1]
        for m in range(Nchi):
            if olist[m, 0] == i and olist[m, 1] == j:
                out[l] = m + 1
                break
    return out


def get_chi_map_soc(olist, invs):
    """Exchange map chi_1234 = sgn chi*_{-4-3-2-1} with spin flips
    (fchi0withsoc.f90:216-279); irr holds 0-based (l, m)."""
    olist = np.asarray(olist)
    inv = np.asarray(invs)
    Nchi = len(olist)
    chi_map = np.zeros((Nchi, Nchi, 2), dtype=np.int64)
    irr_flag = np.zeros((Nchi, Nchi), dtype=bool)
    for l1 in range(Nchi):
        for m1 in range(Nchi):
            t1 = (olist[l1, 0], olist[l1, 1], olist[m1, 0], olist[m1, 1])
            done = False
            for l2 in range(Nchi):
                for m2 in range(Nchi):
                    t2 = (inv[olist[m2, 1] - 1], inv[olist[m2, 0] - 1], inv[olist[l2, 1] - 1],
                          inv[olist[l2, 0] - 1])
                    if t1 == t2:
                        chi_map[m1, l1] = (m2, l2)
                        if not irr_flag[m2, l2]:
                            irr_flag[m1, l1] = True
                        done = True
                        break
                if done:
                    break
    irr = [(l1, m1) for l1 in range(Nchi) for m1 in range(Nchi) if irr_flag[m1, l1]]
    return chi_map, irr


# --------------------------------------------------------------------------- #
#  chi0, vertex, Sigma
# --------------------------------------------------------------------------- #
def pad_green_soc(grid: KGrid, G, a, b, invs, slist):
    """Padded element (a, b) with the spin-orbit time-reversal partner at -k:
    G_ab(-k, iw) = s_a s_b G_{b' a'}(k, iw), primes = spin partners
    (fchi0withsoc.f90:63-78, fselfwithsoc.f90:612-624)."""
    Nw = G.shape[1]
    inv = np.asarray(invs) - 1
    sg = float(slist[a] * slist[b])
    out = grid.empty(2 * Nw)
    rev = (2 * Nw - 1 - np.arange(Nw))[None, :]
    d = grid.flag == 0
    gx, gy, gz, ki = grid.gx[d], grid.gy[d], grid.gz[d], grid.ki[d]
    out[gx, gy, gz, :Nw] = G[ki, :, a, b]
    out[gx[:, None], gy[:, None], gz[:, None], rev] = np.conj(G[ki, :, b, a])
    n = ~d
    gx, gy, gz, ki = grid.gx[n], grid.gy[n], grid.gz[n], grid.ki[n]
    out[gx, gy, gz, :Nw] = sg * G[ki, :, inv[b], inv[a]]
    out[gx[:, None], gy[:, None], gz[:, None], rev] = sg * np.conj(G[ki, :, inv[a], inv[b]])
    return out


def get_chi0_conv_soc(G, grid: KGrid, olist, invs, slist, temp):
    """fchi0withsoc.f90:1-109: per irreducible pair, threshold, then the
    exchange partner set to sgnsig2 * conj."""
    olist = np.asarray(olist)
    Nk, Nw, No, _ = G.shape
    Nchi = len(olist)
    Nkall = len(grid.ki)
    weight = temp / Nkall
    _, sg2 = sign_tables(olist, slist)
    chi_map, irr = get_chi_map_soc(olist, invs)
    chi = np.zeros((Nk, Nw, Nchi, Nchi), dtype=np.complex128)
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    for (l, m) in irr:
        A = np.fft.fftn(pad_green_soc(grid, G, o1[l], o1[m], invs, slist))
        B = np.fft.fftn(pad_green_soc(grid, G, o2[m], o2[l], invs, slist))
        tmp = np.fft.ifftn(-A * _reverse_all(B))
        v = grid.gather_irr(tmp, Nw) * weight
        chi0_threshold(v)
        chi[:, :, m, l] = v
        m2, l2 = chi_map[m, l]
        chi[:, :, m2, l2] = sg2[m, l] * np.conj(chi[:, :, m, l])
    return chi


def ckchi_soc(chi, V_F):
    """max over irreducible q of max Re eig(-chi0(q, nu=0) V) (fchi0withsoc.f90:156-198)."""
    M = -(chi[:, 0] @ V_F)
    return float(np.linalg.eigvals(M).real.max())


def v_soc_flex(chi, V_F):
    """-V + V (I + chi0 V)^-1 chi0 V per (q, nu) (fUJ.f90:367-399)."""
    n = V_F.shape[0]
    X = chi @ V_F
    R = np.linalg.solve(np.eye(n) + X, X)
    return -V_F + V_F @ R


def calc_sigma_soc(G, Vs, V_F, grid: KGrid, olist, invs, slist, temp):
    """fselfwithsoc.f90:540-667: static slot -V(m,l), spin-orbit G pads."""
    olist = np.asarray(olist)
    Nk, Nw, No, _ = G.shape
    Nchi = len(olist)
    Nkall = len(grid.ki)
    sig = np.zeros_like(G)
    Ghat = {}
    for l in range(Nchi):
        for m in range(Nchi):
            W = np.fft.fftn(pad_boson(Vs, grid, m, l, -V_F[m, l]))
            key = (olist[m, 1] - 1, olist[l, 1] - 1)
            if key not in Ghat:
                Ghat[key] = np.fft.fftn(pad_green_soc(grid, G, key[0], key[1], invs, slist))
            tmp = np.fft.ifftn(W * Ghat[key])
            sig[:, :, olist[m, 0] - 1, olist[l, 0] - 1] += grid.gather_irr(tmp, Nw)
    sig *= temp / Nkall
    chi0_threshold(sig)
    return sig


def mkself_soc(V_F, kmap, invk, invs, olist, slist, H_F, eig, U_F, mu_init, fill, temp, scf_loop, pp, eps,
               Nx, Ny, Nz, Nw, sub_sigma=1, m_diis=5, sw_rescale=False, sigma_in=None, mu_old_in=None,
               sigma_scale=1.0):
    """FLEX loop with spin-orbit coupling (fselfwithsoc.f90:1-153).  The loop
    (DIIS compare_sigma, renew_mu with its bracket cache, HF subtraction) is
    the one of fself.f90; n(mu) is computed there from Tr G, equal to the
    eigenvalue sum of the non-SOC get_rn."""
    grid = KGrid(kmap, invk, Nx, Ny, Nz)
    hooks = dict(
        chi=lambda G, mu: get_chi0_conv_soc(G, grid, olist, invs, slist, temp),
        stoner=lambda chi: ckchi_soc(chi, V_F),
        vertex=lambda chi: v_soc_flex(chi, V_F),
        sigma=lambda G, V: calc_sigma_soc(G, V, V_F, grid, olist, invs, slist, temp),
    )
    return mkself(None, None, kmap, invk, olist, H_F, eig, U_F, mu_init, fill, temp, scf_loop, pp, eps,
                  Nx, Ny, Nz, Nw, sub_sigma=sub_sigma, m_diis=m_diis, sw_rescale=sw_rescale, sw_tail=False,
                  sigma_in=sigma_in, mu_old_in=mu_old_in, sigma_scale=sigma_scale, hooks=hooks)


# --------------------------------------------------------------------------- #
#  linearized Eliashberg on the full k mesh
# --------------------------------------------------------------------------- #
def mkfk_trs_soc(G, delta, slist, invk, invs, gap_sym):
    """F(k) = -G(k) Delta(k) G(-k)^H on the full mesh with the spin-orbit TRS
    partner, then the reference's spin-block fills (feliashwithsoc.f90:426-518)."""
    Nk, Nw, No, _ = G.shape
    invk = np.asarray(invk)
    s = np.asarray(slist, dtype=np.float64)
    inv = np.asarray(invs) - 1
    ss = np.outer(s, s)
    ki, flag = invk[:, 0] - 1, invk[:, 1]
    Gk = G[ki]                                                # [Nkall, Nw, No, No]
    Gp = Gk[:, :, inv][:, :, :, inv]                          # G_{l' n'}
    g1 = np.where((flag == 0)[:, None, None, None], Gk, ss[None, None] * np.swapaxes(Gp, -1, -2))
    g2 = np.where((flag == 0)[:, None, None, None], ss[None, None] * Gp, np.swapaxes(Gk, -1, -2))
    F = -(g1 @ delta @ np.conj(np.swapaxes(g2, -1, -2)))
    for l in range(No):
        if s[l] != 1:
            continue
        for m in range(No):
            if s[m] == 1:
                if gap_sym < 0:
                    F[:, :, inv[l], inv[m]] = -np.conj(F[:, :, m, l])
                else:
                    F[:, :, m, l] = 0.0
                    F[:, :, inv[l], inv[m]] = 0.0
            elif inv[m] == l:
                F[:, :, inv[l], inv[m]] = F[:, :, m, l].real
    for l in range(No):
        if s[l] != 1:
            continue
        for m in range(No):
            if s[m] != -1:
                continue
            if gap_sym == -10:
                continue
            F[:, :, inv[m], inv[l]] = F[:, :, m, l] if gap_sym < 0 else -F[:, :, m, l]
    return F


def pad_boson_soc_delta(Vd, grid: KGrid, m, l, static_val, sg2, invschi):
    """Pairing-vertex pad of mkdelta_soc (feliashwithsoc.f90:548-574): at -q the
    spin-flipped pair with the sign sgnsig2(m,l)."""
    Nw = Vd.shape[1]
    out = grid.empty(2 * Nw)
    isl, ism = invschi[l] - 1, invschi[m] - 1
    neg = (2 * Nw - np.arange(1, Nw))[None, :]
    d = grid.flag == 0
    gx, gy, gz, ki = grid.gx[d], grid.gy[d], grid.gz[d], grid.ki[d]
    out[gx, gy, gz, :Nw] = Vd[ki, :, m, l]
    out[gx[:, None], gy[:, None], gz[:, None], neg] = np.conj(Vd[ki, 1:, l, m])
    n = ~d
    gx, gy, gz, ki = grid.gx[n], grid.gy[n], grid.gz[n], grid.ki[n]
    out[gx, gy, gz, :Nw] = sg2 * Vd[ki, :, isl, ism]
    out[gx[:, None], gy[:, None], gz[:, None], neg] = sg2 * np.conj(Vd[ki, 1:, ism, isl])
    out[:, :, :, Nw] = static_val
    return out


def mkdelta_soc(F, Vd, V_F, grid: KGrid, olist, slist, invs, gap_sym):
    """Delta_new(k) = sum V F by FFT convolution on the full mesh, then the
    reference's spin-block fills (feliashwithsoc.f90:520-663); unnormalized."""
    olist = np.asarray(olist)
    Nkall, Nw, No, _ = F.shape
    Nchi = len(olist)
    s = np.asarray(slist)
    inv = np.asarray(invs) - 1
    _, sg2 = sign_tables(olist, slist)
    invschi = get_invschi(olist, invs)
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    mk = np.asarray(grid.invk)[:, 2] - 1
    gx, gy, gz = grid.gx, grid.gy, grid.gz
    rev = (2 * Nw - 1 - np.arange(Nw))[None, :]
    out = np.zeros_like(F)
    for l in range(Nchi):
        for m in range(Nchi):
            mixed = s[o1[l]] * s[o2[m]] < 0
            if not (gap_sym < 0 or (gap_sym > 0 and mixed)):
                continue
            if not ((gap_sym == -10 and mixed) or s[o1[l]] == 1):
                continue
            if not (s[o2[m]] == 1 or o1[l] >= inv[o2[m]]):
                continue
            W = np.fft.fftn(pad_boson_soc_delta(Vd, grid, m, l, -V_F[m, l], sg2[m, l], invschi))
            T = grid.empty(2 * Nw)
            T[gx, gy, gz, :Nw] = F[:, :, o2[l], o1[m]]
            T[gx[:, None], gy[:, None], gz[:, None], rev] = -F[mk, :, o1[m], o2[l]]
            tmp = np.fft.ifftn(W * np.fft.fftn(T))
            out[:, :, o1[l], o2[m]] += tmp[gx, gy, gz, :Nw]
    for l in range(No):
        if s[l] != 1:
            continue
        for m in range(No):
            if s[m] == 1:
                out[:, :, inv[l], inv[m]] = -np.conj(out[:, :, m, l])
            elif inv[m] == l:
                out[:, :, l, m] = out[:, :, l, m].real
            elif l > inv[m]:
                out[:, :, inv[m], inv[l]] = np.conj(out[:, :, l, m])
    for l in range(No):
        if s[l] != 1:
            continue
        for m in range(No):
            if s[m] != -1:
                continue
            if gap_sym > 0:
                out[:, :, inv[l], inv[m]] = -out[:, :, l, m]
            elif gap_sym != -10:
                out[:, :, inv[l], inv[m]] = out[:, :, l, m]
    return out


def get_initial_delta_soc(init_delta_F, U_F, slist, invk, invs, Nw, gap_sym):
    """Band gap phi_n(k) to the orbital basis on the full mesh with the
    spin-orbit partner (feliashwithsoc.f90:665-748), normalized by
    sqrt(2 sum |Delta|^2)."""
    invk = np.asarray(invk)
    s = np.asarray(slist, dtype=np.float64)
    inv = np.asarray(invs) - 1
    Nkall = len(invk)
    No = U_F.shape[1]
    d0 = np.zeros((Nkall, No, No), dtype=np.complex128)
    for i in range(Nkall):
        k, fl = invk[i, 0] - 1, invk[i, 1]
        U = U_F[k]                                            # U[a, n] = uni(a, n, k)
        if fl == 0:
            L = U * init_delta_F[k][None, :]
            R = (s[None, :] * np.conj(U[inv, :]).T)           # R[n, l] = s_l conj uni(l', n)
            d0[i] = -(L @ R)
        elif fl == 1:
            L = (s[:, None] * np.conj(U[inv, :])) * init_delta_F[k][None, :]
            d0[i] = L @ U.T
        if gap_sym > 0:
            d0[i][np.outer(s, s) >= 0] = 0.0
    d = np.repeat(d0[:, None], Nw, axis=1)
    return d / np.sqrt(2.0 * np.sum(np.abs(d) ** 2))


class LinEliashSocResult:
    def __init__(self, delta, lam, ritz1=None, ritz2=None):
        self.delta, self.lam, self.ritz1, self.ritz2 = delta, lam, ritz1, ritz2


def lin_eliash_soc(chi, G, U_F, init_delta_F, V_F, olist, slist, kmap, invk, invs, temp, eps, Nx, Ny, Nz,
                   itemax, gap_sym, arnoldi_m):
    """feliashwithsoc.f90:1-424: V_Delta = -V + V chi V (chi overwritten), then
    the two-pass Arnoldi or the shifted power method on the full-mesh gap with
    A v = -(T/Nkall) mkdelta_soc(mkfk_trs_soc(v)) and <u,v> = 2 sum conj(u) v."""
    grid = KGrid(kmap, invk, Nx, Ny, Nz)
    Nk, Nw = G.shape[:2]
    Nkall = len(grid.ki)
    weight = temp / Nkall
    Vd = v_soc_flex(chi, V_F)

    def apply_op(v):
        return -mkdelta_soc(mkfk_trs_soc(G, v, slist, invk, invs, gap_sym), Vd, V_F, grid, olist, slist, invs,
                            gap_sym) * weight

    def inner(u, v):
        return 2.0 * np.sum(np.conj(u) * v)

    def norm(f):
        return float(np.sqrt(2.0 * np.sum(np.abs(f) ** 2)))

    def init():
        return get_initial_delta_soc(init_delta_F, U_F, slist, invk, invs, Nw, gap_sym)

    if arnoldi_m <= 0:
        return _power_soc(apply_op, inner, norm, init, eps, itemax), Vd

    def arnoldi(v0, shift, defl):
        V = [v0]
        H = np.zeros((arnoldi_m + 1, arnoldi_m), dtype=np.complex128)
        m_act = arnoldi_m
        for j in range(arnoldi_m):
            w = apply_op(V[j])
            if shift is not None:
                w = w + shift * V[j]
                w = w - inner(defl, w) * defl
            for ii in range(j + 1):
                h = inner(V[ii], w)
                H[ii, j] = h
                w = w - h * V[ii]
            beta = norm(w)
            H[j + 1, j] = beta
            if beta < 1e-14:
                m_act = j + 1
                break
            if j < arnoldi_m - 1:
                V.append(w * (1.0 / beta))
        ev, vr = np.linalg.eig(H[:m_act, :m_act])
        return V, ev, vr, m_act

    def ritz(V, vr, idx, m_act):
        y = _zgeev_vector(vr[:, idx])
        d = np.zeros_like(V[0])
        for ii in range(m_act):
            d = d + y[ii] * V[ii]
        return d * (1.0 / norm(d))

    V, ev, vr, m_act = arnoldi(init(), None, None)
    idx = int(np.argmin(ev.real))
    lam1 = float(ev[idx].real)
    if ev.real.max() >= 0.1:
        idx = int(np.argmax(ev.real))
        return LinEliashSocResult(ritz(V, vr, idx, m_act), float(ev[idx].real), ev), Vd
    delta1 = ritz(V, vr, idx, m_act)
    shift = -lam1
    v0 = init()
    v0 = v0 - inner(delta1, v0) * delta1
    v0 = v0 * (1.0 / norm(v0))
    V2, ev2, vr2, m_act2 = arnoldi(v0, shift, delta1)
    idx = int(np.argmax(ev2.real))
    return LinEliashSocResult(ritz(V2, vr2, idx, m_act2), float(ev2[idx].real) - shift, ev, ev2), Vd


def _power_soc(apply_op, inner, norm, init, eps, itemax):
    """Shifted power method of lin_eliash_soc (feliashwithsoc.f90:60-110):
    pass 2 runs with the shift |newdelta| of pass 1 and no deflation."""
    norm2 = 0.0
    newdelta = None
    lam = 0.0
    for i_eig in (1, 2):
        delta = init()
        count = 0
        nrm = 1.0
        for it in range(1, itemax + 1):
            newdelta = apply_op(delta) + delta * norm2
            nrm = norm(newdelta)
            inrm = 1.0 / nrm
            lam_rq = float(inner(delta, newdelta).real)
            vp = np.sum(np.abs(newdelta * inrm - delta) ** 2)
            vn = np.sum(np.abs(newdelta * inrm + delta) ** 2)
            verr = float(np.sqrt(2.0 * min(vp, vn)))
            lam = lam_rq - norm2
            if verr < eps:
                if lam > 0.1 or lam < 0.0:
                    break
                if verr < eps * 1e-2:
                    count += 1
                if count > 30:
                    break
            delta = newdelta * inrm
        if i_eig == 1 and lam > 0.0:
            break
        norm2 = nrm
    return LinEliashSocResult(newdelta * (1.0 / norm(newdelta)), lam)


def conv_delta_orb_to_band_soc(delta, U_F, invk, invs, slist):
    """Orbital-basis gap at the first Matsubara frequency to the band basis
    (feliashwithsoc.f90:750-794); delta on the full mesh."""
    invk = np.asarray(invk)
    s = np.asarray(slist, dtype=np.float64)
    inv = np.asarray(invs) - 1
    Nkall, _, No, _ = delta.shape
    out = np.zeros((Nkall, No, No), dtype=np.complex128)
    for i in range(Nkall):
        k, fl = invk[i, 0] - 1, invk[i, 1]
        U = U_F[k]
        if fl == 0:
            L = np.conj(U).T
            R = s[:, None] * U[inv, :]
        elif fl == 1:
            L = (-s[None, :]) * U[inv, :].T
            R = np.conj(U)
        else:
            continue
        out[i] = L @ delta[i, 0] @ R
    return out


def get_chis_chic_soc(chi, V_F, orb_list, olist, slist):
    """nu = 0 RPA with spin-orbit coupling, X = (I + chi0 V)^-1 chi0, summed into
    charge, S_zz and S+- channels by spin labels (fchi0withsoc.f90:281-326)."""
    olist = np.asarray(olist)
    s = np.asarray(slist)
    Nk, Nw, Nchi, _ = chi.shape
    n4 = Nchi // 4
    c0 = chi[:, 0]
    X = np.linalg.solve(np.eye(Nchi) + c0 @ V_F, c0)
    chic = np.zeros((Nk, n4, n4), dtype=np.complex128)
    chiszz = np.zeros_like(chic)
    chispm = np.zeros_like(chic)
    ol = np.asarray(orb_list) - 1
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    for l in range(Nchi):
        for m in range(Nchi):
            if s[o1[l]] == s[o1[m]] and s[o2[l]] == s[o2[m]]:
                if s[o1[l]] == -s[o2[l]] and s[o1[l]] == 1:
                    chispm[:, ol[l], ol[m]] += X[:, m, l]
            if s[o1[l]] == s[o2[l]] and s[o1[m]] == s[o2[m]]:
                chic[:, ol[l], ol[m]] += X[:, m, l]
                if s[o1[l]] == s[o1[m]]:
                    chiszz[:, ol[l], ol[m]] += X[:, m, l]
                else:
                    chiszz[:, ol[l], ol[m]] -= X[:, m, l]
    return chic * 0.5, chiszz * 0.25, chispm


def gen_green0_soc(eig, U_F, mu, temp, Nw):
    return gen_green0_F(eig, U_F, mu, temp, Nw)


def gen_green_soc(sigma_F, H_F, mu, temp):
    return gen_green_F(sigma_F, H_F, mu, temp)


__all__ = ["get_vmat_soc", "sign_tables", "get_invschi", "get_chi_map_soc", "pad_green_soc",
           "get_chi0_conv_soc", "ckchi_soc", "v_soc_flex", "calc_sigma_soc", "mkself_soc", "mkfk_trs_soc",
           "mkdelta_soc", "get_initial_delta_soc", "lin_eliash_soc", "conv_delta_orb_to_band_soc",
           "get_chis_chic_soc", "hf_subtract", "matsubara"]
