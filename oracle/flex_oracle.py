"""CPU FP64 restatement of the pyrpa FLEX / RPA / linearized-Eliashberg hot path.

THIS MODULE IS TEST INFRASTRUCTURE.  It is the checker for the CUDA engine in
``pyrpa_gb300`` and is imported only by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product never calls it.

It restates, in NumPy and in FP64/complex128, the Fortran routines of the
reference ``libfmod.so`` that the FLEX / Eliashberg path runs (ktszk/pyrpa,
``libs/src/*.f90``).  Each function names the file:line range it follows.
The reference cannot be compiled here (no Fortran compiler), so the oracle is
pinned by the reference's own known-answer tests (``tests/test_rpa_flex.py``,
``tests/test_tools.py`` and the exact references of ``tests/_tools.py``),
which ``tests/test_oracle_reference_kat.py`` re-states against this module.
Converged Sigma / lambda of a non-trivial model are not pinned by any
reference test: for those the oracle is a restatement, parity unpinned
beyond the known-answer tests.

Conventions.  Arrays handled inside this module use the *Fortran view*: a
0-based NumPy array whose index order equals the Fortran dummy's index order,
e.g. ``G[i, j, a, b]`` is Fortran ``Gk(i+1, j+1, a+1, b+1)`` with shape
``(Nk, Nw, Norb, Norb)``.  The pyrpa Python wrappers hand C-ordered arrays of
the reversed shape to the library, so ``G_fortran_view = Gk_python.T``.
``kmap``/``invk`` are used in the Python shape ``(Nkall, 3)`` (1-based irr
index in ``invk[:, 0]``) and ``olist`` as ``(Nchi, 2)`` with 1-based orbitals.
"""
from __future__ import annotations

import numpy as np

PI = 3.141592653589793238462643383279


# --------------------------------------------------------------------------- #
#  k mesh with time-reversal reduction (finv.f90:1-305, _hamiltonian.py:356-382)
# --------------------------------------------------------------------------- #
def irr_k_count(Nx: int, Ny: int, Nz: int) -> int:
    """Irreducible k count used by gen_irr_k_TRS (libs/flibs/_hamiltonian.py:367-378)."""
    Nkall = Nx * Ny * Nz
    if Nkall % 2 == 0:
        if Nz % 2 == 0:
            if Nx % 2 == 0 and Ny % 2 == 0:
                return Nkall // 2 + 4
            if Nx % 2 == 0 or Ny % 2 == 0:
                return Nkall // 2 + 2
            return Nkall // 2 + 1
        if Nx % 2 == 0 and Ny % 2 == 0:
            return Nkall // 2 + 2
        return Nkall // 2 + 1
    return (Nkall + 1) // 2


def _irr_k_grid(Nx: int, Ny: int, Nz: int, Nk: int) -> np.ndarray:
    """Integer grid coordinates of the irreducible list, in the reference's
    order (finv.f90:117-288, gen_irr_k).  Slots use the reference's 1-based
    ``iter_k`` arithmetic; unfilled slots stay (0,0,0) as in the Fortran."""
    kl = np.zeros((Nk, 3), dtype=np.int64)

    def put(it, i, j, k=0):
        kl[it - 1] = (i, j, k)

    def half_plane(ini, k):
        # one kz plane reduced by inversion; returns next free 1-based slot
        if Nx % 2 == 0 and Ny % 2 == 0:
            for j in range(Ny // 2 + 1):
                for i in range(Nx // 2 + 1):
                    put(ini + i + (Nx // 2 + 1) * j, i, j, k)
            ini2 = ini + (Nx // 2 + 1) * (Ny // 2 + 1) - 1
            for j in range(Ny // 2 + 1, Ny):
                for i in range(1, Nx // 2):
                    put(ini2 + i + (Nx // 2 - 1) * (j - Ny // 2 - 1), i, j, k)
            return ini + Nx * Ny // 2 + 2
        it = ini
        if (Nx * Ny) % 2 == 0:
            if Nx % 2 != 0:
                raise ValueError("odd Nx with even Ny: the reference irreducible list "
                                 "is undefined for this mesh (finv.f90:143-166)")
            for j in range((Ny - 1) // 2 + 1):
                for i in range(Nx // 2 + 1):
                    put(it, i, j, k)
                    it += 1
            for j in range((Ny + 1) // 2, Ny):
                for i in range(1, Nx // 2):
                    put(it, i, j, k)
                    it += 1
            return it
        for j in range((Ny - 1) // 2 + 1):
            for i in range((Nx - 1) // 2 + 1):
                put(it, i, j, k)
                it += 1
        for j in range((Ny + 1) // 2, Ny):
            for i in range(1, (Nx - 1) // 2 + 1):
                put(it, i, j, k)
                it += 1
        return it

    ini = half_plane(1, 0)
    if Nz > 1:
        nfull = Nz // 2 - 1 if Nz % 2 == 0 else (Nz - 1) // 2
        for k in range(1, nfull + 1):
            for j in range(Ny):
                for i in range(Nx):
                    put(ini + i + Nx * j + Nx * Ny * (k - 1), i, j, k)
        ini += Nx * Ny * nfull
        if Nz % 2 == 0:
            half_plane(ini, Nz // 2)
    return kl


def generate_irr_kpoint_inv(Nx: int, Ny: int, Nz: int):
    """(klist[Nk,3], kmap[Nkall,3], invk[Nkall,3]) as gen_irr_k_TRS returns them
    (finv.f90:1-67).  invk[:,0]: 1-based irreducible index, invk[:,1]: 0 direct /
    1 via -k, invk[:,2]: 1-based full index of -k.  The reference compares
    fractional coordinates with a tolerance 1/max(N); on grid points that is
    equality of integer coordinates, which is what is used here."""
    Nk = irr_k_count(Nx, Ny, Nz)
    Nkall = Nx * Ny * Nz
    irr = _irr_k_grid(Nx, Ny, Nz, Nk)
    dims = np.array([Nx, Ny, Nz])
    klist = irr / dims
    x, y, z = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    kmap = np.stack([x.ravel(order="F"), y.ravel(order="F"), z.ravel(order="F")], axis=1)
    kmap = kmap.astype(np.int64)
    direct, inverse = {}, {}
    for j, c in enumerate(irr):
        direct.setdefault(tuple(c), j)
        inverse.setdefault(tuple((-c) % dims), j)
    invk = np.zeros((Nkall, 3), dtype=np.int64)
    for g in range(Nkall):
        c = tuple(kmap[g])
        jd, ji = direct.get(c), inverse.get(c)
        if jd is None and ji is None:
            raise ValueError("k point without irreducible partner")
        if jd is not None and (ji is None or jd <= ji):
            invk[g, 0], invk[g, 1] = jd + 1, 0
        else:
            invk[g, 0], invk[g, 1] = ji + 1, 1
        m = (-kmap[g]) % dims
        invk[g, 2] = m[0] + Nx * (m[1] + Ny * m[2]) + 1
    return klist, kmap, invk


def get_kweight(invk: np.ndarray, Nk: int) -> np.ndarray:
    """Multiplicity of each irreducible k (finv.f90:292-305)."""
    return np.bincount(invk[:, 0] - 1, minlength=Nk).astype(np.float64)


# --------------------------------------------------------------------------- #
#  band structure (fmod.f90:162-248, 312-340, 657-716)
# --------------------------------------------------------------------------- #
def gen_ham_F(klist: np.ndarray, ham_r_py: np.ndarray, rvec: np.ndarray) -> np.ndarray:
    """H_F[i, m, l] = Fortran ham_k(m,l,i): lower triangle summed, then made
    Hermitian (fmod.f90:162-207).  ham_r_py is the Python [Nr,Norb,Norb] array."""
    HrF = np.transpose(ham_r_py, (0, 2, 1))            # HrF[j, m, l] = ham_r(m,l,j)
    ph = 2 * PI * klist @ rvec.T                       # [Nk, Nr]
    cph = np.cos(ph) - 1j * np.sin(ph)
    H = np.einsum("kr,rml->kml", cph, HrF)
    No = H.shape[1]
    out = np.zeros_like(H)
    for l in range(No):
        out[:, l, l] = H[:, l, l].real
        for m in range(l + 1, No):
            out[:, m, l] = H[:, m, l]
            out[:, l, m] = np.conj(H[:, m, l])
    return out


def get_eig_F(H_F: np.ndarray):
    """(eig[Nk,Norb], U_F[Nk,Norb,Norb]) with U_F[i,:,n] the n-th eigenvector
    (fmod.f90:209-248).  Eigenvector phases follow numpy, not zheev."""
    w, v = np.linalg.eigh(H_F)
    return w, v


def _upper_hermitian(A):
    """The Hermitian matrix zheev('V','U') sees: A's upper triangle."""
    return np.triu(A) + np.conj(np.swapaxes(np.triu(A, 1), -1, -2))


def get_eig_mlo_F(H_F: np.ndarray, S_F: np.ndarray):
    """(eig[Nk,Norb], U_F[Nk,Norb,Norb]) in a non-orthogonal basis by canonical
    orthogonalization (fmod.f90:250-310): S = V_s diag(s) V_s^H, X = V_s
    diag(1/sqrt(s)) with the columns of s <= 1e-8 zeroed, H_orth = X^H H X,
    H_orth = V diag(e) V^H, U = X V.  Eigenvector phases follow numpy."""
    s, Vs = np.linalg.eigh(_upper_hermitian(S_F))
    keep = s > 1.0e-8
    X = Vs * np.where(keep, 1.0 / np.sqrt(np.where(keep, s, 1.0)), 0.0)[:, None, :]
    Ho = _upper_hermitian(np.conj(np.swapaxes(X, -1, -2)) @ (H_F @ X))
    e, V = np.linalg.eigh(Ho)
    return e, X @ V


def get_ffermi(eig: np.ndarray, mu: float, temp: float) -> np.ndarray:
    """fmod.f90:312-340."""
    t = max(temp, 1e-12)
    return 0.5 - 0.5 * np.tanh((eig - mu) * (0.5 / t))


def get_parity_prop(rvec: np.ndarray, ham_r_py: np.ndarray) -> np.ndarray:
    """Pmn (Fortran view) of orbital parities, +1/-1 (fmod.f90:657-716)."""
    Nr = len(rvec)
    HrF = np.transpose(ham_r_py, (0, 2, 1))
    No = HrF.shape[1]
    num = np.zeros((No, No))
    den = np.zeros((No, No))
    for i in range(Nr):
        for j in range(i + 1, Nr):
            if np.abs(rvec[i] + rvec[j]).sum() < 1e-6:
                num += (HrF[j] * np.conj(HrF[i])).real
                den += np.abs(HrF[i]) ** 2
                break
    P = np.where(den > 1e-10, num / np.where(den > 1e-10, den, 1.0), 0.0)
    return np.where(P >= 0.0, 1.0, -1.0)


# --------------------------------------------------------------------------- #
#  interaction vertices (fUJ.f90:1-107)
# --------------------------------------------------------------------------- #
def get_scmat(olist: np.ndarray, site: np.ndarray, U: float, J: float):
    """Python-layout Smat, Cmat [Nchi,Nchi]: entry [i,j] is the rule evaluated
    at loop indices (i,j) of fUJ.f90:33-55 (stored there as Smat(j,i))."""
    Nchi = len(olist)
    Up = U - 2 * J
    S = np.zeros((Nchi, Nchi))
    C = np.zeros((Nchi, Nchi))
    for i in range(Nchi):
        for j in range(Nchi):
            if site[i] != site[j]:
                continue
            oi, oj = olist[i], olist[j]
            if oi[0] == oi[1] and oj[0] == oj[1]:
                if oi[0] == oj[0]:
                    S[i, j], C[i, j] = U, U
                else:
                    S[i, j], C[i, j] = J, 2 * Up - J
            elif oi[0] == oj[0] and oi[1] == oj[1]:
                S[i, j], C[i, j] = Up, -Up + 2 * J
            elif oi[0] == oj[1] and oi[1] == oj[0]:
                S[i, j], C[i, j] = J, J
    return S, C


def get_scmat_orb(olist, site, Umat_py, Jmat_py):
    """Orbital-dependent variant (fUJ.f90:59-107); Umat_py/Jmat_py are Python
    [Norb,Norb] so Fortran Umat(a,b) = Umat_py[b-1,a-1]."""
    Nchi = len(olist)
    UF = lambda a, b: Umat_py[b - 1, a - 1]
    JF = lambda a, b: Jmat_py[b - 1, a - 1]
    S = np.zeros((Nchi, Nchi))
    C = np.zeros((Nchi, Nchi))
    for i in range(Nchi):
        for j in range(Nchi):
            if site[i] != site[j]:
                continue
            oi, oj = olist[i], olist[j]
            if oi[0] == oi[1] and oj[0] == oj[1]:
                if oi[0] == oj[0]:
                    S[i, j] = C[i, j] = UF(oi[0], oi[0])
                else:
                    S[i, j] = JF(oi[0], oj[0])
                    C[i, j] = 2 * UF(oi[0], oj[0]) - JF(oi[0], oj[0])
            elif oi[0] == oj[0] and oi[1] == oj[1]:
                S[i, j] = UF(oi[0], oi[1])
                C[i, j] = -UF(oi[0], oi[1]) + 2 * JF(oi[0], oi[1])
            elif oi[0] == oj[1] and oi[1] == oj[0]:
                S[i, j] = C[i, j] = JF(oi[0], oi[1])
    return S, C


def get_chi_orb_list(Norb: int, site_prof=(1,)):
    """Orbital-pair list and site labels as plibs.get_chi_orb_list builds
    them (libs/plibs/_response.py:382-413).  Within a site of ns orbitals
    starting at orbital f, pair l = (f + l % ns, f + l // ns); one site spans
    all orbitals with label 1, several sites are labelled by their first
    orbital.  A profile that does not add up to Norb is refused (the
    reference prints and exits)."""
    prof = [int(x) for x in site_prof]
    if len(prof) > 1 and sum(prof) != Norb:
        raise SystemExit("site_prof doesn't correspond to Hamiltonian")
    sites = [Norb] if len(prof) == 1 else prof
    pairs, labels, first = [], [], 1
    for ns in sites:
        l = np.arange(ns * ns)
        pairs.append(np.stack([first + l % ns, first + l // ns], axis=1))
        labels.append(np.full(ns * ns, 1 if len(prof) == 1 else first))
        first += ns
    return np.concatenate(pairs).astype(np.int64), np.concatenate(labels).astype(np.int64)


# --------------------------------------------------------------------------- #
#  Green functions (fself.f90:1-157)
# --------------------------------------------------------------------------- #
def matsubara(temp: float, Nw: int) -> np.ndarray:
    return (2 * np.arange(Nw) + 1) * PI * temp


def gen_green0_F(eig, U_F, mu, temp, Nw):
    """G0[i,j,m,l] = sum_n U(m,n) U*(l,n) / (mu + i w_j - e_n)  (fself.f90:1-41)."""
    iw = mu + 1j * matsubara(temp, Nw)
    den = 1.0 / (iw[None, :, None] - eig[:, None, :])          # [Nk,Nw,n]
    return np.einsum("kmn,kln,kwn->kwml", U_F, np.conj(U_F), den)


def gen_green_F(sigma_F, H_F, mu, temp):
    """G = (i w + mu - H - Sigma)^-1 per (k,w)  (fself.f90:43-157)."""
    Nk, Nw, No, _ = sigma_F.shape
    iw = mu + 1j * matsubara(temp, Nw)
    A = -(H_F[:, None, :, :] + sigma_F)
    A = A + iw[None, :, None, None] * np.eye(No)[None, None]
    return np.linalg.inv(A)


def gen_green_inv_from_eig_F(sigma_F, eig, U_F, mu, temp):
    """G^-1[i,j,m,l] = sum_n U(m,n) U*(l,n) (mu + i w_j - e_n) - Sigma[i,j,m,l]
    with the U given, unitary or not (fself.f90:85-129)."""
    iw = mu + 1j * matsubara(temp, sigma_F.shape[1])
    fac = iw[None, :, None] - eig[:, None, :]                   # [Nk,Nw,n]
    return np.einsum("kmn,kln,kwn->kwml", U_F, np.conj(U_F), fac) - sigma_F


# --------------------------------------------------------------------------- #
#  chi0 (fchi.f90:319-918)
# --------------------------------------------------------------------------- #
def get_chi_map(olist: np.ndarray):
    """(chi_map[m,l] -> (m2,l2) 0-based, irr list of (l,m) 0-based) following
    fchi.f90:421-481.  chi_1234 = chi*_4321 with 1234 = (o(l,1),o(l,2),o(m,1),o(m,2))."""
    Nchi = len(olist)
    chi_map = np.zeros((Nchi, Nchi, 2), dtype=np.int64)
    chi_irr = np.zeros((Nchi, Nchi), dtype=bool)
    for l1 in range(Nchi):
        for m1 in range(Nchi):
            t1 = (olist[l1, 0], olist[l1, 1], olist[m1, 0], olist[m1, 1])
            done = False
            for l2 in range(Nchi):
                for m2 in range(Nchi):
                    t2 = (olist[m2, 1], olist[m2, 0], olist[l2, 1], olist[l2, 0])
                    if t1 == t2:
                        chi_map[m1, l1] = (m2, l2)
                        if not chi_irr[m2, l2]:
                            chi_irr[m1, l1] = True
                        done = True
                        break
                if done:
                    break
    irr = [(l1, m1) for l1 in range(Nchi) for m1 in range(Nchi) if chi_irr[m1, l1]]
    return chi_map, irr


class KGrid:
    """Index helpers for the full grid (x fastest) built from kmap/invk."""

    def __init__(self, kmap, invk, Nx, Ny, Nz):
        self.Nx, self.Ny, self.Nz = Nx, Ny, Nz
        self.kmap = np.asarray(kmap)
        self.invk = np.asarray(invk)
        self.ki = self.invk[:, 0] - 1
        self.flag = self.invk[:, 1]
        self.gx, self.gy, self.gz = self.kmap[:, 0], self.kmap[:, 1], self.kmap[:, 2]
        self.direct = np.where(self.flag == 0)[0]

    def empty(self, M):
        return np.zeros((self.Nx, self.Ny, self.Nz, M), dtype=np.complex128)

    def pad_green(self, G, a, b):
        """Full-grid padded array of element (a,b) (0-based): slot j<Nw holds
        G_ab(k,iw_j), slot 2Nw-1-j holds conj G_ba(k,iw_j); at -k the TRS
        partner is used (fchi.f90:563-583)."""
        Nw = G.shape[1]
        out = self.empty(2 * Nw)
        d = self.flag == 0
        for sel, (p, q) in ((d, (a, b)), (~d, (b, a))):
            gx, gy, gz, ki = self.gx[sel], self.gy[sel], self.gz[sel], self.ki[sel]
            out[gx, gy, gz, :Nw] = G[ki, :, p, q]
            out[gx[:, None], gy[:, None], gz[:, None], (2 * Nw - 1 - np.arange(Nw))[None, :]] = np.conj(G[ki, :, q, p])
        return out

    def gather_irr(self, full, Nw):
        """values at irreducible k (via the direct full-grid point), slots < Nw."""
        Nk = self.ki.max() + 1
        out = np.zeros((Nk, Nw), dtype=np.complex128)
        d = self.direct
        np.add.at(out, self.ki[d], full[self.gx[d], self.gy[d], self.gz[d], :Nw])
        return out


def _reverse_all(a):
    """a(-x,-y,-z,-n) with indices taken modulo each axis length."""
    for ax in range(a.ndim):
        a = np.roll(np.flip(a, axis=ax), 1, axis=ax)
    return a


def _reverse_space(a):
    for ax in range(3):
        a = np.roll(np.flip(a, axis=ax), 1, axis=ax)
    return a


def chi0_conv_acc(chi, G, grid: KGrid, olist, temp, coef, chi_map, irr):
    """chi += coef * bubble (fchi.f90:508-613).  Adds then sets the exchange
    partner to the conjugate, exactly in the reference's order."""
    Nk, Nw = G.shape[0], G.shape[1]
    Nkall = len(grid.ki)
    weight = coef * temp / Nkall
    for (l, m) in irr:
        A = np.fft.fftn(grid.pad_green(G, olist[l, 0] - 1, olist[m, 0] - 1))
        B = np.fft.fftn(grid.pad_green(G, olist[m, 1] - 1, olist[l, 1] - 1))
        tmp = np.fft.ifftn(-A * _reverse_all(B))
        chi[:, :, m, l] += grid.gather_irr(tmp, Nw) * weight
        m2, l2 = chi_map[m, l]
        chi[:, :, m2, l2] = np.conj(chi[:, :, m, l])


def chi0_threshold(chi, eps=1.0e-9):
    """fchi.f90:483-506."""
    re = np.where(np.abs(chi.real) < eps, 0.0, chi.real)
    im = np.where(np.abs(chi.imag) < eps, 0.0, chi.imag)
    chi[...] = re + 1j * im


def get_chi0_conv(G, grid, olist, temp):
    """fchi.f90:615-635."""
    Nk, Nw = G.shape[:2]
    Nchi = len(olist)
    chi = np.zeros((Nk, Nw, Nchi, Nchi), dtype=np.complex128)
    chi_map, irr = get_chi_map(olist)
    chi0_conv_acc(chi, G, grid, olist, temp, 1.0, chi_map, irr)
    chi0_threshold(chi)
    return chi


def chi0_ref_tau(chi, eig, U_F, mu, grid: KGrid, olist, temp, Nw, chi_map, irr):
    """Analytic tau-space reference bubble added into chi (fchi.f90:637-850)."""
    Nkall = len(grid.ki)
    M = 2 * Nw
    beta = 1.0 / temp
    dtau = beta / M
    weight = 1.0 / (temp * Nkall)
    xi = eig - mu                                       # [Nk, n]
    tau = np.arange(M) * dtau
    pos = xi >= 0
    e_pb = np.exp(-beta * np.abs(xi))                   # exp(-beta|xi|)
    ff = np.where(pos, e_pb / (1 + e_pb), 1.0 / (1 + e_pb))
    gp = np.where(pos[..., None], -np.exp(-xi[..., None] * tau) / (1 + e_pb[..., None]),
                  -np.exp(xi[..., None] * (beta - tau)) / (1 + e_pb[..., None]))
    gm = np.where(pos[..., None], np.exp(-xi[..., None] * (beta - tau)) / (1 + e_pb[..., None]),
                  np.exp(xi[..., None] * tau) / (1 + e_pb[..., None]))
    # gp, gm: [Nk, n, s]
    rho = np.einsum("kmn,kln,kn->kml", U_F, np.conj(U_F), ff)
    rhobar = np.zeros(rho.shape[1:], dtype=np.complex128)
    for g in range(Nkall):
        if grid.flag[g] == 0:
            rhobar += rho[grid.ki[g]]
        elif grid.flag[g] == 1:
            rhobar += rho[grid.ki[g]].T
    rhobar /= Nkall
    s = np.arange(M)
    sawc = np.zeros(Nw, dtype=np.complex128)
    for j in range(Nw):
        if j > 0:
            sawc[j] = 1j / (2.0 * PI * j * temp)
        ph = np.exp(1j * 2.0 * PI * j * s / M)
        sawc[j] -= dtau * np.sum(ph * (0.5 - s / M))
    d = grid.flag == 0
    for (l, m) in irr:
        a13, b13 = olist[l, 0] - 1, olist[m, 0] - 1
        a42, b42 = olist[m, 1] - 1, olist[l, 1] - 1
        U13 = U_F[:, a13, :] * np.conj(U_F[:, b13, :])      # [Nk, n]
        U42 = U_F[:, a42, :] * np.conj(U_F[:, b42, :])
        A = grid.empty(M)
        B = grid.empty(M)
        for sel, cj in ((d, False), (~d, True)):
            ki = grid.ki[sel]
            u13 = np.conj(U13[ki]) if cj else U13[ki]
            u42 = np.conj(U42[ki]) if cj else U42[ki]
            A[grid.gx[sel], grid.gy[sel], grid.gz[sel]] = np.einsum("kn,kns->ks", u13, gp[ki])
            B[grid.gx[sel], grid.gy[sel], grid.gz[sel]] = np.einsum("kn,kns->ks", u42, gm[ki])
        A = np.fft.fftn(A, axes=(0, 1, 2))
        B = np.fft.fftn(B, axes=(0, 1, 2))
        tmp = np.fft.ifftn(-A * _reverse_space(B))
        J = 0.0j
        if a13 == b13:
            J += rhobar[a42, b42]
        if a42 == b42:
            J -= rhobar[a13, b13]
        chi[:, :, m, l] += grid.gather_irr(tmp, Nw) * weight + J * sawc[None, :]
        m2, l2 = chi_map[m, l]
        chi[:, :, m2, l2] = np.conj(chi[:, :, m, l])


def chi0_tail(G, eig, U_F, mu, grid, olist, temp):
    """chi0 = conv[G] - conv[G0] + analytic reference (fchi.f90:852-892)."""
    Nk, Nw = G.shape[:2]
    Nchi = len(olist)
    chi = np.zeros((Nk, Nw, Nchi, Nchi), dtype=np.complex128)
    chi_map, irr = get_chi_map(olist)
    chi0_conv_acc(chi, G, grid, olist, temp, 1.0, chi_map, irr)
    G0 = gen_green0_F(eig, U_F, mu, temp, Nw)
    chi0_conv_acc(chi, G0, grid, olist, temp, -1.0, chi_map, irr)
    chi0_ref_tau(chi, eig, U_F, mu, grid, olist, temp, Nw, chi_map, irr)
    chi0_threshold(chi)
    return chi


def ckchi(chi, S_F, C_F):
    """(max_q max Re eig(chi0(q,0) S), same for -chi0 C, q index of each)
    (fchi.f90:352-399)."""
    X = chi[:, 0]
    es = np.linalg.eigvals(X @ S_F).real.max(axis=1)
    ec = np.linalg.eigvals(-X @ C_F).real.max(axis=1)
    return float(es.max()), float(ec.max()), int(es.argmax()), int(ec.argmax())


def get_chis_F(chi0_F, S_F):
    """chis = (I - chi0 S)^-1 chi0 per slice (fchi.f90:319-350).  chi0_F[i] is
    the Fortran-view matrix of slice i."""
    n = S_F.shape[0]
    A = np.eye(n)[None] - chi0_F @ S_F
    return np.linalg.solve(A, chi0_F)


def get_chis_chic_F(chi, S_F, C_F):
    """(chis, chic)[k] at nu=0 (fself.f90:783-816)."""
    X = chi[:, 0]
    n = S_F.shape[0]
    chis = np.linalg.solve(np.eye(n)[None] - X @ S_F, X)
    chic = np.linalg.solve(np.eye(n)[None] + X @ C_F, X)
    return chis, chic


def get_eig_or_tr_chi(chiq_F, invk, sw_eig):
    """Full-grid max Re eigenvalue or trace (fself.f90:818-851)."""
    ki = invk[:, 0] - 1
    if sw_eig:
        vals = np.linalg.eigvals(chiq_F).real.max(axis=1).astype(np.complex128)
    else:
        vals = np.trace(chiq_F, axis1=1, axis2=2)
    return vals[ki]


def vsigma_flex_nosoc(chi, S_F, C_F):
    """V_sigma per (q,iw) (fUJ.f90:318-365)."""
    n = S_F.shape[0]
    I = np.eye(n)
    XS = chi @ S_F
    XC = chi @ C_F
    Xs = np.linalg.solve(I - XS, XS)
    Xc = np.linalg.solve(I + XC, XC)
    SC = S_F + C_F
    return (1.5 * S_F - 0.5 * C_F) + 1.5 * (S_F @ Xs) + 0.5 * (C_F @ Xc) - 0.25 * (SC @ (XS + XC))


def vdelta_nsoc_flex(chi, S_F, C_F, singlet: bool):
    """V_Delta per (q,iw) (fUJ.f90:253-316)."""
    n = S_F.shape[0]
    I = np.eye(n)
    XS = chi @ S_F
    XC = chi @ C_F
    Xs = np.linalg.solve(I - XS, XS)
    Xc = np.linalg.solve(I + XC, XC)
    if singlet:
        return 0.5 * (S_F + C_F) + 1.5 * (S_F @ Xs) - 0.5 * (C_F @ Xc)
    return 0.5 * (S_F - C_F) - 0.5 * (S_F @ Xs) - 0.5 * (C_F @ Xc)


# --------------------------------------------------------------------------- #
#  self-energy (fself.f90:159-285)
# --------------------------------------------------------------------------- #
def pad_boson(V, grid: KGrid, m, l, static_val):
    """Padded bosonic array of pair (m,l) (fself.f90:201-223): slot 0 = nu_0,
    slots 1..Nw-1 = nu_j, slot Nw = static value, slot 2Nw-j = conj V_lm(nu_j)."""
    Nw = V.shape[1]
    out = grid.empty(2 * Nw)
    d = grid.flag == 0
    for sel, (p, q) in ((d, (m, l)), (~d, (l, m))):
        gx, gy, gz, ki = grid.gx[sel], grid.gy[sel], grid.gz[sel], grid.ki[sel]
        out[gx, gy, gz, :Nw] = V[ki, :, p, q]
        out[gx[:, None], gy[:, None], gz[:, None], (2 * Nw - np.arange(1, Nw))[None, :]] = np.conj(V[ki, 1:, q, p])
    out[:, :, :, Nw] = static_val
    return out


def calc_sigma(G, V, S_F, C_F, grid: KGrid, olist, temp):
    """fself.f90:159-285."""
    Nk, Nw, No, _ = G.shape
    Nchi = len(olist)
    Nkall = len(grid.ki)
    sig = np.zeros_like(G)
    Ghat = {}
    for l in range(Nchi):
        for m in range(Nchi):
            W = np.fft.fftn(pad_boson(V, grid, m, l, 1.5 * S_F[m, l] - 0.5 * C_F[m, l]))
            key = (olist[m, 1] - 1, olist[l, 1] - 1)
            if key not in Ghat:
                Ghat[key] = np.fft.fftn(grid.pad_green(G, *key))
            tmp = np.fft.ifftn(W * Ghat[key])
            sig[:, :, olist[m, 0] - 1, olist[l, 0] - 1] += grid.gather_irr(tmp, Nw)
    sig *= temp / Nkall
    chi0_threshold(sig)
    return sig


def hf_subtract(sig, mode=1):
    """fself.f90:384-416."""
    Nk, Nw, No, _ = sig.shape
    sub = np.zeros((Nk, No, No), dtype=np.complex128)
    for l in range(No):
        for m in range(l, No):
            if mode == 1:
                v = (sig[:, 0, l, m] + np.conj(sig[:, 0, m, l])) * 0.5
            else:
                v = np.sum(sig[:, :, l, m] + np.conj(sig[:, :, m, l]), axis=1) * (0.5 / Nw)
            sub[:, l, m] = v
            if l != m:
                sub[:, m, l] = np.conj(v)
    return sig - sub[:, None]


# --------------------------------------------------------------------------- #
#  FLEX loop (fself.f90:287-781)
# --------------------------------------------------------------------------- #
class MkselfResult:
    def __init__(self, sigma, mu, iterations, esterr, stoner, history):
        self.sigma, self.mu, self.iterations = sigma, mu, iterations
        self.esterr, self.stoner, self.history = esterr, stoner, history


def mkself(S_F, C_F, kmap, invk, olist, H_F, eig, U_F, mu_init, fill, temp, scf_loop,
           pp, eps, Nx, Ny, Nz, Nw, sub_sigma=1, m_diis=5, sw_rescale=True,
           sw_tail=False, sigma_in=None, mu_old_in=None, sigma_scale=1.0, verbose=False, hooks=None):
    """FLEX self-consistency loop, restated from fself.f90:287-446 with
    compare_sigma (:449-542), renew_mu (:544-660), get_rn (:662-687) and
    precompute_eig_gkinv (:689-711).  sigma_in/mu_old_in emulate sw_in.
    hooks (chi, stoner, vertex, sigma) replace the four physics steps; the
    spin-orbit loop of fselfwithsoc.f90 passes its own."""
    grid = KGrid(kmap, invk, Nx, Ny, Nz)
    Nk = H_F.shape[0]
    No = H_F.shape[1]
    wl = matsubara(temp, Nw)
    mu = mu_init
    st = dict(mu_old=mu * 1.2, n_hist=0, i_hist=0, bracket=None, esterr=0.0)
    if sigma_in is not None:
        sig = sigma_in.copy() * (sigma_scale if sigma_scale != 1.0 else 1.0)
        st["mu_old"] = mu_old_in
        sig0 = sig.copy()
        G = gen_green_F(sig, H_F, mu, temp)
    else:
        sig = np.zeros((Nk, Nw, No, No), dtype=np.complex128)
        sig0 = sig.copy()
        G = gen_green0_F(eig, U_F, mu, temp, Nw)
    xout = [None] * m_diis
    res = [None] * m_diis
    history = []
    eig_g = None

    def get_rn(rmu):
        t = np.sum(0.5 * (1.0 - np.tanh(0.5 * (eig - rmu) / temp)))
        z = rmu + 1j * wl
        dg = np.sum((1.0 / (z[None, :, None] - eig_g) - 1.0 / (z[None, :, None] - eig[:, None, :])).real)
        return (t + 2 * temp * dg) / Nk

    def renew_mu():
        nonlocal mu, eig_g
        eig_g = np.linalg.eigvals(H_F[:, None] + sig)       # [Nk, Nw, n]
        e = 1e-8 if st["esterr"] > 1e-2 else st["esterr"] * 0.1
        dmu = abs(mu - st["mu_old"]) * 2.0
        if dmu < e * 4.0:
            dmu = e * 4.0
        st["mu_old"] = mu
        found = False
        if st["bracket"] is not None:
            mS, mL = st["bracket"]
            rS, rL = get_rn(mS), get_rn(mL)
            if rS < fill and rL > fill:
                muS, muL, rnS, rnL = mS, mL, rS, rL
                found = True
        if not found:
            muL, muS = mu + dmu, mu - dmu
            for it in range(1, 101):
                mu = muL
                rnL = get_rn(mu)
                if rnL < fill:
                    if abs(fill - rnL) > 0.5:
                        muL += 1.0
                    elif abs(fill - rnL) > dmu:
                        muL += 0.5
                    else:
                        muL += dmu
                else:
                    break
                if it == 100:
                    raise RuntimeError("Too many")
            for it in range(1, 101):
                mu = muS
                rnS = get_rn(mu)
                if rnS > fill:
                    if abs(rnS - fill) > 0.5:
                        muS -= 1.0
                    elif abs(rnS - fill) > dmu:
                        muS -= 0.5
                    else:
                        muS -= dmu
                else:
                    break
                if it == 100:
                    raise RuntimeError("Too many")
        st["bracket"] = (muS, muL)
        rnL -= fill
        rnS -= fill
        rnc, muc, mud, flag = rnS, muS, 0.0, False
        for it in range(1, 101):
            if rnc != rnS and rnc != rnL:
                muM = (muL * rnS * rnc * (rnS - rnc) + muS * rnL * rnc * (rnc - rnL)
                       + muc * rnL * rnS * (rnL - rnS)) / ((rnL - rnS) * (rnc - rnL) * (rnc - rnS))
            else:
                muM = muL - rnL * (muL - muS) / (rnL - rnS)
            if ((0.25 * (3.0 * muS + muL) > muM or muM > muL)
                    or (flag and abs(muM - muL) >= abs(muL - muc) * 0.5)
                    or ((not flag) and abs(muM - muL) >= abs(muc - mud) * 0.5)
                    or (flag and abs(muL - muc) < 1.0e-8)
                    or ((not flag) and abs(muc - mud) < 1.0e-8)):
                muM = (muL + muS) * 0.5
                flag = True
            else:
                flag = False
            if abs(muL - muM) < e:
                break
            mu = muM
            rnM = get_rn(muM)
            mud, muc, rnc = muc, muL, rnL
            if rnS * (rnM - fill) < 0:
                muL, rnL = muM, rnM - fill
            else:
                muS, rnS = muM, rnM - fill
            if abs(rnS) < abs(rnL):
                muL, muS = muS, muL
                rnL, rnS = rnS, rnL
            if it == 100:
                raise RuntimeError("Too many loop!")
        mu = (muS + muL) * 0.5 if rnL == rnS else (muS * rnL - muL * rnS) / (rnL - rnS)
        st["mu_old"] = mu

    def compare_sigma():
        nonlocal sig
        st["i_hist"] = st["i_hist"] % m_diis + 1
        st["n_hist"] = min(st["n_hist"] + 1, m_diis)
        ih = st["i_hist"] - 1
        xout[ih] = sig.copy()
        res[ih] = sig - sig0
        n = st["n_hist"]
        idx = [((st["i_hist"] - n + h - 1) % m_diis) for h in range(1, n + 1)]
        B = np.zeros((n + 1, n + 1))
        for a, ia in enumerate(idx):
            for b, ib in enumerate(idx):
                B[a, b] = np.sum(np.conj(res[ia]) * res[ib]).real
            B[a, n] = B[n, a] = 1.0
        for a in range(n):
            B[a, a] += 1e-12
        rhs = np.zeros(n + 1)
        rhs[n] = 1.0
        try:
            c = np.linalg.solve(B, rhs)
        except np.linalg.LinAlgError:
            c = np.zeros(n + 1)
            c[n - 1] = 1.0
        sd = np.zeros_like(sig)
        for a, ia in enumerate(idx):
            sd = sd + c[a] * xout[ia]
        mask = np.abs(sd) > 1e-10
        est = np.abs((sig0 - sd) / np.where(mask, sd, 1.0))
        st["esterr"] = float(est[mask].max()) if mask.any() else 0.0
        sig = sd if n >= 2 else pp * sd + (1.0 - pp) * sig0

    stoner = 0.0
    it_done = 0
    for scf_i in range(1, scf_loop + 1):
        it_done = scf_i
        if hooks is not None:
            chi = hooks["chi"](G, mu)
            stoner = hooks["stoner"](chi)
        elif sw_tail:
            chi = chi0_tail(G, eig, U_F, mu, grid, olist, temp)
        else:
            chi = get_chi0_conv(G, grid, olist, temp)
        if hooks is None:
            stoner = ckchi(chi, S_F, C_F)[0]
        if sw_rescale and stoner >= 1.0:
            chi = chi * ((1.0 - 1.0e-4) / stoner)
        if hooks is not None:
            sig = hooks["sigma"](G, hooks["vertex"](chi))
        else:
            V = vsigma_flex_nosoc(chi, S_F, C_F)
            sig = calc_sigma(G, V, S_F, C_F, grid, olist, temp)
        if sub_sigma > 0:
            sig = hf_subtract(sig, sub_sigma)
        compare_sigma()
        history.append(dict(esterr=st["esterr"], mu=mu, stoner=stoner))
        if verbose:
            print(f"iter={scf_i} esterr={st['esterr']:.3e} mu={mu:.8f} stoner={stoner:.6f}")
        if st["esterr"] < eps:
            break
        renew_mu()
        G = gen_green_F(sig, H_F, mu, temp)
        sig0 = sig.copy()
    renew_mu()
    return MkselfResult(sig, mu, it_done, st["esterr"], stoner, history)


# --------------------------------------------------------------------------- #
#  linearized Eliashberg (feliash.f90:1-821)
# --------------------------------------------------------------------------- #
def mkfk_F(G, delta):
    """F = -G Delta G^H, then Hermitian form (feliash.f90:445-484)."""
    F = -(G @ delta @ np.conj(np.swapaxes(G, -1, -2)))
    return hermitize_lower(F)


def hermitize_lower(A):
    """diag real, upper triangle = conj of lower (feliash.f90:473-481)."""
    A = A.copy()
    n = A.shape[-1]
    for l in range(n):
        A[..., l, l] = A[..., l, l].real
        for m in range(l + 1, n):
            A[..., l, m] = np.conj(A[..., m, l])
    return A


def mkdelta_nsoc(F, Vd, S_F, C_F, grid: KGrid, prt, olist, singlet: bool):
    """Delta_new = sum V F by FFT convolution, unnormalized (feliash.f90:486-635)."""
    Nk, Nw, No, _ = F.shape
    Nchi = len(olist)
    sgn = 1.0 if singlet else -1.0
    dprt = 1.0 if singlet else -1.0
    out = np.zeros_like(F)
    d = grid.flag == 0
    for l in range(Nchi):
        for m in range(Nchi):
            if olist[l, 0] < olist[m, 1]:
                continue
            W = pad_boson(Vd, grid, m, l, 0.5 * (S_F[m, l] + sgn * C_F[m, l]))
            a, b = olist[l, 1] - 1, olist[m, 0] - 1
            pp_ = prt[a] * prt[b]
            T = grid.empty(2 * Nw)
            rev = 2 * Nw - 1 - np.arange(Nw)
            for sel, inv in ((d, False), (~d, True)):
                gx, gy, gz, ki = grid.gx[sel], grid.gy[sel], grid.gz[sel], grid.ki[sel]
                if not inv:
                    T[gx, gy, gz, :Nw] = F[ki, :, a, b]
                    T[gx[:, None], gy[:, None], gz[:, None], rev[None, :]] = sgn * dprt * pp_ * np.conj(F[ki, :, a, b])
                else:
                    T[gx, gy, gz, :Nw] = pp_ * dprt * F[ki, :, a, b]
                    T[gx[:, None], gy[:, None], gz[:, None], rev[None, :]] = sgn * F[ki, :, b, a]
            tmp = np.fft.ifftn(np.fft.fftn(W) * np.fft.fftn(T))
            out[:, :, olist[l, 0] - 1, olist[m, 1] - 1] += grid.gather_irr(tmp, Nw)
    return hermitize_upper_from_lower(out)


def hermitize_upper_from_lower(A):
    """feliash.f90:618-634: for l<m, A[l,m] = conj A[m,l]; diag real."""
    return hermitize_lower(A)


def get_initial_delta(init_delta_F, U_F, invk, Nw, gap_sym):
    """feliash.f90:637-731.  init_delta_F[i,n] = Fortran init_delta(i,n)."""
    Nk, No = init_delta_F.shape
    if gap_sym == 0:
        d = np.zeros((Nk, Nw, No, No), dtype=np.complex128)
        for l in range(No):
            d[:, :, l, l] = 1.0
    else:
        tmpu = U_F * init_delta_F[:, None, :]
        d0 = hermitize_lower(tmpu @ np.conj(np.swapaxes(U_F, -1, -2)))
        d = np.repeat(d0[:, None], Nw, axis=1).astype(np.complex128)
    w = get_kweight(invk, Nk)
    nrm = np.sum(w[:, None, None, None] * np.abs(d) ** 2)
    if nrm <= 0:
        raise RuntimeError("get_initial_delta norm <= 0")
    return d / np.sqrt(2.0 * nrm)


def _zgeev_vector(vec):
    """Unit 2-norm with the largest-magnitude component real (LAPACK zgeev)."""
    vec = vec / np.linalg.norm(vec)
    k = int(np.argmax(np.abs(vec)))
    return vec * (np.conj(vec[k]) / abs(vec[k]))


class LinEliashResult:
    def __init__(self, delta, lam, ritz1, ritz2):
        self.delta, self.lam, self.ritz1, self.ritz2 = delta, lam, ritz1, ritz2


def lin_eliash(chi, G, U_F, init_delta_F, S_F, C_F, olist, prt, kmap, invk, temp, eps,
               Nx, Ny, Nz, itemax, gap_sym, arnoldi_m, arnoldi_tol=0.0):
    """feliash.f90:1-443 (V_Delta, then Arnoldi two-pass or shifted power method).
    arnoldi_tol > 0 (the engine's pyrpa_gb_set_arnoldi_tol, not in the
    reference) restarts the pass that gives lambda from its Ritz vector,
    arnoldi_m steps at a time and at most 12 cycles, until the Ritz residual
    |h_{m+1,m} y_m| / |lambda| is below the tolerance."""
    grid = KGrid(kmap, invk, Nx, Ny, Nz)
    Nk, Nw = G.shape[:2]
    Nkall = len(grid.ki)
    singlet = gap_sym >= 0
    weight = temp / Nkall
    kw = get_kweight(invk, Nk)[:, None, None, None]
    Vd = vdelta_nsoc_flex(chi, S_F, C_F, singlet)

    def apply_op(v):
        return mkdelta_nsoc(mkfk_F(G, v), Vd, S_F, C_F, grid, prt, olist, singlet) * weight

    def inner(u, v):
        return 2.0 * np.sum(kw * np.conj(u) * v)

    def norm(f):
        return float(np.sqrt(2.0 * np.sum(kw * np.abs(f) ** 2)))

    init = lambda: get_initial_delta(init_delta_F, U_F, invk, Nw, gap_sym)

    if arnoldi_m <= 0:
        return _power_method(apply_op, inner, norm, init, eps, itemax, Vd)

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
        return V, ev, vr, m_act, H

    def ritz(V, vr, idx, m_act):
        y = _zgeev_vector(vr[:, idx])
        d = np.zeros_like(V[0])
        for ii in range(m_act):
            d = d + y[ii] * V[ii]
        return d * (1.0 / norm(d))

    def residual(H, vr, idx, m_act):
        y = vr[:, idx]
        return abs(H[m_act, m_act - 1]) * abs(y[m_act - 1]) / np.linalg.norm(y)

    def converge(V, ev, vr, m_act, H, shift, defl):
        s0 = 0.0 if shift is None else shift
        idx = int(np.argmax(ev.real))
        d, lam, res, cycles = ritz(V, vr, idx, m_act), float(ev[idx].real) - s0, residual(H, vr, idx, m_act), 1
        while arnoldi_tol > 0 and res > arnoldi_tol * abs(lam) and cycles < 12:
            V, ev, vr, m_act, H = arnoldi(d, shift, defl)
            idx = int(np.argmax(ev.real))
            d, lam, res = ritz(V, vr, idx, m_act), float(ev[idx].real) - s0, residual(H, vr, idx, m_act)
            cycles += 1
        return d, lam, ev

    V, ev, vr, m_act, H = arnoldi(init(), None, None)
    idx = int(np.argmin(ev.real))
    lam1 = float(ev[idx].real)
    if ev.real.max() >= 0.1:
        d, lam, ev = converge(V, ev, vr, m_act, H, None, None)
        return LinEliashResult(d, lam, ev, None)
    delta1 = ritz(V, vr, idx, m_act)
    shift = -lam1
    v0 = init()
    v0 = v0 - inner(delta1, v0) * delta1
    b = norm(v0)
    if b < 1e-14:
        return LinEliashResult(delta1, lam1, ev, None)
    v0 = v0 * (1.0 / b)
    V2, ev2, vr2, m_act2, H2 = arnoldi(v0, shift, delta1)
    d, lam, ev2 = converge(V2, ev2, vr2, m_act2, H2, shift, delta1)
    return LinEliashResult(d, lam, ev, ev2)


def _power_method(apply_op, inner, norm, init, eps, itemax, Vd):
    """Shifted power method with deflation (feliash.f90:66-140)."""
    lam_out = 0.0
    lambda1 = 0.0
    delta1 = None
    newdelta = None
    for i_eig in (1, 2):
        delta = init()
        if i_eig == 2:
            proj = inner(delta1, delta).real
            delta = delta - proj * delta1
            delta = delta * (1.0 / norm(delta))
        lam_prev = 0.0
        lam_rq = lam_phys = 0.0
        for it in range(1, itemax + 1):
            newdelta = apply_op(delta)
            if i_eig == 2:
                newdelta = newdelta - lambda1 * delta
                proj = inner(delta1, newdelta).real
                newdelta = newdelta - proj * delta1
            nrm = norm(newdelta)
            if nrm <= 0:
                raise RuntimeError("norm <= 0")
            inrm = 1.0 / nrm
            lam_rq = inner(delta, newdelta).real
            lam_phys = lam_rq + lambda1
            vp = np.sqrt(max(0.0, (norm(newdelta * inrm - delta)) ** 2))
            vn = np.sqrt(max(0.0, (norm(newdelta * inrm + delta)) ** 2))
            verr = min(vp, vn)
            if lam_phys < 0 and verr < eps:
                break
            if verr < eps and abs(lam_phys - lam_prev) < eps * (abs(lam_phys) + 1e-10):
                break
            lam_prev = lam_phys
            delta = newdelta * inrm
        if i_eig == 1:
            if lam_phys > 0:
                lam_out = lam_phys
                break
            lambda1 = lam_rq
            delta1 = newdelta * inrm
        else:
            lam_out = lam_phys
    return LinEliashResult(newdelta * (1.0 / norm(newdelta)), lam_out, None, None)


def conv_delta_orb_to_band_F(delta, U_F, prt, invk, gap_sym):
    """Band-basis gap at w_0 on the full grid (feliash.f90:733-785)."""
    Nkall = len(invk)
    No = U_F.shape[1]
    dprt = -1.0 if gap_sym < 0 else 1.0
    out = np.zeros((Nkall, No, No), dtype=np.complex128)
    for i in range(Nkall):
        k = invk[i, 0] - 1
        if invk[i, 1] == 0:
            out[i] = np.conj(U_F[k].T) @ delta[k, 0] @ U_F[k]
        elif invk[i, 1] == 1:
            L = U_F[k].T * prt[None, :]
            tm = (L @ delta[k, 0]) * (dprt * prt)[None, :]
            out[i] = tm @ np.conj(U_F[k])
    return out


def remap_delta_F(delta0, prt, invk, gap_sym):
    """Full-grid gap from the irreducible one (feliash.f90:787-821)."""
    dprt = -1.0 if gap_sym < 0 else 1.0
    ki = invk[:, 0] - 1
    out = delta0[ki].copy()
    inv = invk[:, 1] == 1
    out[inv] *= dprt * prt[None, None, :, None] * prt[None, None, None, :]
    return out


# --------------------------------------------------------------------------- #
#  Sigma seed regrid along the Matsubara axis (libs/plibs/_calc.py:52-182)
# --------------------------------------------------------------------------- #
def _spline_uniform_notaknot(y, h):
    """Second derivatives M of the not-a-knot cubic spline through y on a
    uniform grid of spacing h, along axis 1 (scipy's CubicSpline default
    boundary condition, restated on the uniform grid: the not-a-knot rows make
    M_1 and M_{n-2} explicit, the interior is tridiagonal)."""
    n = y.shape[1]
    r = np.zeros_like(y)
    r[:, 1:-1] = 6.0 * (y[:, 2:] - 2.0 * y[:, 1:-1] + y[:, :-2]) / (h * h)
    M = np.zeros_like(y)
    if n < 4:
        return M if n < 3 else np.repeat(r[:, 1:2] / 6.0, 3, axis=1)
    M[:, 1] = r[:, 1] / 6.0
    M[:, n - 2] = r[:, n - 2] / 6.0
    m = n - 4  # unknowns M_2 .. M_{n-3}
    if m > 0:
        d = r[:, 2:n - 2].copy()
        d[:, 0] -= M[:, 1]
        d[:, -1] -= M[:, n - 2]
        # Thomas algorithm for tridiag(1, 4, 1)
        c = np.zeros(m)
        c[0] = 1.0 / 4.0
        d[:, 0] /= 4.0
        for i in range(1, m):
            den = 4.0 - c[i - 1]
            c[i] = 1.0 / den
            d[:, i] = (d[:, i] - d[:, i - 1]) / den
        for i in range(m - 2, -1, -1):
            d[:, i] -= c[i] * d[:, i + 1]
        M[:, 2:n - 2] = d
    M[:, 0] = 2.0 * M[:, 1] - M[:, 2]
    M[:, n - 1] = 2.0 * M[:, n - 2] - M[:, n - 3]
    return M


def regrid_sigma(sig, temp_old, temp_new, Nw_new, w_scale=1.0):
    """Sigma(k, iw_n) of the Matsubara mesh at temp_old (Fortran view
    (Nk, Nw_old, Norb, Norb)) onto Nw_new frequencies at temp_new, as
    plibs.regrid_sigma_bin computes it (libs/plibs/_calc.py:127-171): the
    outermost stored frequency is dropped, the data are extended to negative
    frequencies with Sigma_lm(-iw) = conj Sigma_ml(iw), interpolated by a
    not-a-knot cubic spline in w, extended beyond the kept cutoff by
    c0 + c1/(iw) fitted by least squares over the stored points
    [0.55 n, max(0.85 n, 0.55 n + 4)), and the diagonal clipped to
    Im Sigma_ll <= 0."""
    Nk, Nw_old, No, _ = sig.shape
    s = sig[:, :Nw_old - 1]
    nk = Nw_old - 1
    w_old = (2.0 * np.arange(nk) + 1.0) * PI * temp_old
    w_new = w_scale * (2.0 * np.arange(Nw_new) + 1.0) * PI * temp_new
    mirror = np.conj(np.swapaxes(s, 2, 3))[:, ::-1]
    ext = np.concatenate([mirror, s], axis=1)                  # (Nk, 2nk, No, No)
    wext = np.concatenate([-w_old[::-1], w_old])
    h = 2.0 * PI * temp_old
    y = np.moveaxis(ext, 1, -1).reshape(-1, 2 * nk)            # series along the last axis
    yy = np.concatenate([y.real, y.imag], axis=0)
    M = _spline_uniform_notaknot(yy, h)
    out = np.full((yy.shape[0], Nw_new), np.nan)
    inside = (w_new >= wext[0]) & (w_new <= wext[-1])
    for q in np.where(inside)[0]:
        x = w_new[q]
        i = min(int(np.floor((x - wext[0]) / h)), 2 * nk - 2)
        a, b = wext[i + 1] - x, x - wext[i]
        out[:, q] = (M[:, i] * a ** 3 + M[:, i + 1] * b ** 3) / (6.0 * h) + \
            (yy[:, i] / h - M[:, i] * h / 6.0) * a + (yy[:, i + 1] / h - M[:, i + 1] * h / 6.0) * b
    half = y.shape[0]
    res = (out[:half] + 1j * out[half:]).reshape(Nk, No, No, Nw_new)
    res = np.moveaxis(res, -1, 1).copy()
    beyond = w_new > w_old[-1]
    if beyond.any():
        i0, i1 = int(0.55 * nk), max(int(0.85 * nk), int(0.55 * nk) + 4)
        basis = np.stack([np.ones(i1 - i0), 1.0 / (1j * w_old[i0:i1])], axis=1)
        rhs = s[:, i0:i1].reshape(Nk, i1 - i0, No * No).transpose(1, 0, 2).reshape(i1 - i0, -1)
        coef = np.linalg.lstsq(basis, rhs, rcond=None)[0]
        c0 = coef[0].reshape(Nk, No, No)
        c1 = coef[1].reshape(Nk, No, No)
        res[:, beyond] = c0[:, None] + c1[:, None] / (1j * w_new[beyond])[None, :, None, None]
    di = np.arange(No)
    d = res[:, :, di, di]
    res[:, :, di, di] = d.real + 1j * np.minimum(d.imag, 0.0)
    return res


# --------------------------------------------------------------------------- #
#  Nonlinear FLEX-Eliashberg (ffeliash.f90:1-612)
# --------------------------------------------------------------------------- #
def mkgreliah_F(G0, F, delta):
    """G = G0 (I + Delta F^H) per (k, iw)  (ffeliash.f90:316-343)."""
    No = G0.shape[-1]
    M = delta @ np.conj(np.swapaxes(F, -1, -2)) + np.eye(No)
    return G0 @ M


def mkfkeliash_F(G0, G, delta):
    """F = -G0 Delta G^H, diagonal real, upper = conj(lower)  (ffeliash.f90:345-377)."""
    F = -(G0 @ (delta @ np.conj(np.swapaxes(G, -1, -2))))
    return hermitize_lower(F)


def mkV_flex_sc(XS0, XC0, S_F, C_F, singlet: bool):
    """V_sigma and V_Delta from the spin- and charge-channel chi0 (ffeliash.f90:379-452).
    The double-counting term uses chi0_S S + chi0_C C, as the reference assembles it."""
    n = S_F.shape[0]
    I = np.eye(n)
    P = XS0 @ S_F
    Q = XC0 @ C_F
    X5 = P + Q
    chis = np.linalg.solve(I - P, P)
    chic = np.linalg.solve(I + Q, Q)
    Vs = (1.5 * S_F - 0.5 * C_F) + 1.5 * (S_F @ chis) + 0.5 * (C_F @ chic) - 0.25 * ((S_F + C_F) @ X5)
    if singlet:
        Vd = 0.5 * (S_F + C_F) + 1.5 * (S_F @ chis) - 0.5 * (C_F @ chic)
    else:
        Vd = 0.5 * (S_F - C_F) - 0.5 * (S_F @ chis) - 0.5 * (C_F @ chic)
    return Vs, Vd


def get_chi0_conv_ff(F, grid: KGrid, olist, prt, temp, singlet: bool):
    """chi^FF bubble by FFT convolution (ffeliash.f90:491-612).  At -k the
    reference reads F(olist(m,1), olist(l,1)) for the +iw leg of F^+14 and
    F(olist(l,2), olist(m,2)) for F23 (where +k reads olist(m,2) / olist(m,1));
    that is restated as it is."""
    Nk, Nw, No, _ = F.shape
    Nchi = len(olist)
    Nkall = len(grid.ki)
    sgn = dprt = 1.0 if singlet else -1.0
    weight = temp / Nkall
    chi = np.zeros((Nk, Nw, Nchi, Nchi), dtype=np.complex128)
    chi_map, irr = get_chi_map(olist)
    o1, o2 = olist[:, 0] - 1, olist[:, 1] - 1
    rev = 2 * Nw - 1 - np.arange(Nw)
    d = grid.flag == 0
    for (l, m) in irr:
        A = grid.empty(2 * Nw)
        B = grid.empty(2 * Nw)
        pa = prt[o1[l]] * prt[o2[m]] * sgn * dprt
        pb = prt[o1[m]] * prt[o2[l]] * sgn * dprt
        for sel, inv in ((d, False), (~d, True)):
            gx, gy, gz, ki = grid.gx[sel], grid.gy[sel], grid.gz[sel], grid.ki[sel]
            ix = (gx[:, None], gy[:, None], gz[:, None], rev[None, :])
            if not inv:
                A[gx, gy, gz, :Nw] = np.conj(F[ki, :, o2[m], o1[l]])
                B[gx, gy, gz, :Nw] = F[ki, :, o2[l], o1[m]]
                A[ix] = pa * np.conj(F[ki, :, o1[l], o2[m]])
                B[ix] = pb * F[ki, :, o1[m], o2[l]]
            else:
                A[gx, gy, gz, :Nw] = np.conj(F[ki, :, o1[m], o1[l]])
                B[gx, gy, gz, :Nw] = F[ki, :, o2[l], o2[m]]
                A[ix] = pa * np.conj(F[ki, :, o1[l], o2[m]])
                B[ix] = pb * F[ki, :, o2[l], o1[m]]
        tmp = np.fft.ifftn(-np.fft.fftn(A) * _reverse_all(np.fft.fftn(B)))
        v = grid.gather_irr(tmp, Nw) * weight
        v = np.where(np.abs(v.real) < 1e-9, 0.0, v.real) + 1j * np.where(np.abs(v.imag) < 1e-9, 0.0, v.imag)
        chi[:, :, m, l] = v
        m2, l2 = chi_map[m, l]
        chi[:, :, m2, l2] = np.conj(chi[:, :, m, l])
    return chi


def get_chi0sc(G, F, grid, olist, prt, temp, singlet):
    """(chi0_S, chi0_C) = chi^GG +- chi^FF  (ffeliash.f90:454-489)."""
    gg = get_chi0_conv(G, grid, olist, temp)
    ff = get_chi0_conv_ff(F, grid, olist, prt, temp, singlet)
    return gg + ff, gg - ff


class NonlinEliashResult:
    def __init__(self, delta, sigma, G, iterations, history):
        self.delta, self.sigma, self.G = delta, sigma, G
        self.iterations, self.history = iterations, history


def nonlinear_eliashberg(delta, sigma, G, H_F, S_F, C_F, olist, prt, kmap, invk, mu, temp, eps, Nx, Ny, Nz,
                         itemax, gap_sym, sw_sigma, sw_Vconst, m_diis, gap_min, sw_amp_newton):
    """Nonlinear FLEX-Eliashberg loop (ffeliash.f90:2-314), Fortran-view arrays."""
    delta, sigma, G = delta.copy(), sigma.copy(), G.copy()
    grid = KGrid(kmap, invk, Nx, Ny, Nz)
    Nkall = len(grid.ki)
    singlet = gap_sym >= 0
    m_eff = max(int(m_diis), 1)
    pp, eps_reg = 0.3, 1.0e-12
    weight = temp / Nkall
    xout = [None] * m_eff
    res = [None] * m_eff
    n_hist = i_hist = 0
    amp_phase, npts, n_polish, n_anchor = 1, 0, 0, 0
    a1 = a2 = g1 = g2 = 0.0
    a_cur = float(np.sqrt(np.sum(np.conj(delta) * delta).real)) + 1.0e-300
    v0 = delta / a_cur
    if not sw_amp_newton:
        amp_phase = 2
    G0 = G.copy()
    delta0_max = np.abs(delta).max() + 1.0e-30
    if sw_Vconst:
        XS, XC = get_chi0sc(G, np.zeros_like(G), grid, olist, prt, temp, singlet)
        F = mkfk_F(G, delta)
    else:
        F = mkfk_F(G, delta)
        XS, XC = get_chi0sc(G, F, grid, olist, prt, temp, singlet)
    Vs, Vd = mkV_flex_sc(XS, XC, S_F, C_F, singlet)
    if not sw_sigma:
        sigma[...] = 0.0
    history = []
    it = 0
    for it in range(1, itemax + 1):
        newdelta = mkdelta_nsoc(F, Vd, S_F, C_F, grid, prt, olist, singlet) * weight
        diff = np.abs(newdelta - delta).max()
        norm = np.abs(delta).max() + 1.0e-30
        new_max = np.abs(newdelta).max()
        history.append(dict(rel=diff / norm, new_max=new_max))
        if diff / norm < eps:
            delta = newdelta
            break
        if gap_min > 0.0 and new_max < gap_min * delta0_max:
            delta = newdelta
            break
        if sw_amp_newton and amp_phase == 2 and n_polish >= 10:
            a_cur = float(np.sqrt(np.sum(np.conj(delta) * delta).real)) + 1.0e-300
            v0 = delta / a_cur
            npts, a1, a2, g1, g2 = 0, 0.0, 0.0, 0.0, 0.0
            amp_phase = 1
            n_anchor += 1
        if amp_phase == 1:
            proj = float(np.sum(np.conj(v0) * newdelta).real)
            g_cur = proj / a_cur
            a2, g2, a1, g1 = a1, g1, a_cur, g_cur
            npts = min(npts + 1, 2)
            if npts >= 2 and abs(a1 * a1 - a2 * a2) > 1.0e-30:
                cfit = (g1 - g2) / (a2 * a2 - a1 * a1)
                lam0 = g1 + cfit * a1 * a1
                if cfit > 1.0e-12 and lam0 > 1.0:
                    a_nxt = float(np.sqrt((lam0 - 1.0) / cfit))
                    a_nxt = min(max(a_nxt, 0.3 * a_cur), 3.0 * a_cur)
                else:
                    a_nxt = 0.5 * a_cur
            else:
                a_nxt = 0.9 * a_cur if abs(g_cur - 1.0) < 0.2 else 0.6 * a_cur
            if abs(g_cur - 1.0) < 2.0e-2:
                amp_phase = 2
                a_nxt = a_cur
                n_polish = 0
                n_hist = i_hist = 0
            history[-1].update(phase=1, a=a_cur, g=g_cur, a_next=a_nxt)
            delta = a_nxt * v0
            a_cur = a_nxt
        else:
            i_hist = i_hist % m_eff + 1
            n_hist = min(n_hist + 1, m_eff)
            n = n_hist
            xout[i_hist - 1] = newdelta.copy()
            res[i_hist - 1] = newdelta - delta
            do_pulay = n >= 2 and m_eff >= 2
            if do_pulay:
                idx = [((i_hist - n + h - 1) % m_eff) for h in range(1, n + 1)]
                B = np.zeros((n + 1, n + 1))
                for a_, ia in enumerate(idx):
                    for b_, ib in enumerate(idx):
                        B[a_, b_] = np.sum(np.conj(res[ia]) * res[ib]).real
                    B[a_, a_] += eps_reg
                    B[a_, n] = B[n, a_] = 1.0
                rhs = np.zeros(n + 1)
                rhs[n] = 1.0
                try:
                    c = np.linalg.solve(B, rhs)
                except np.linalg.LinAlgError:
                    do_pulay = False
            if do_pulay:
                delta = np.zeros_like(delta)
                for a_, ia in enumerate(idx):
                    delta = delta + c[a_] * xout[ia]
            else:
                delta = pp * newdelta + (1.0 - pp) * delta
            n_polish += 1
        if sw_sigma:
            sigma = calc_sigma(G, Vs, S_F, C_F, grid, olist, temp)
            G0 = gen_green_F(sigma, H_F, mu, temp)
        G = mkgreliah_F(G0, F, delta)
        F = mkfkeliash_F(G0, G, delta)
        if not sw_Vconst:
            XS, XC = get_chi0sc(G, F, grid, olist, prt, temp, singlet)
            Vs, Vd = mkV_flex_sc(XS, XC, S_F, C_F, singlet)
    return NonlinEliashResult(delta, sigma, G, it, history)
