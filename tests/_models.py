"""Model builders and exact references shared by the test-suite.

The models are the closed-form square-lattice tight-binding bundles the
reference suite uses (pyrpa ``tests/_tools.py:114-175``); the exact bubble is
the textbook Matsubara Lindhard function with an optional exactly solvable
two-pole self-energy Sigma = a^2/(i w + mu - delta) (``tests/_tools.py:214-283``).
Every array here is in the Python layout the ``flibs`` wrappers use.
"""
from __future__ import annotations

import numpy as np

PI = np.pi


def fermi(e, temp, mu=0.0):
    """Overflow-safe Fermi function."""
    x = np.asarray(e - mu, dtype=np.float64) / temp
    ax = np.abs(x)
    em = np.exp(-ax)
    return np.where(x > 0, em / (1.0 + em), 1.0 / (1.0 + em))


def square_hoppings(tx=1.0, ty=0.5, t2=0.0):
    """Nearest (and optional next-nearest) neighbour one-orbital hoppings."""
    rv = [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]]
    hv = [0.0, -tx, -tx, -ty, -ty]
    if t2 != 0.0:
        rv += [[1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0]]
        hv += [-t2] * 4
    rvec = np.array(rv, dtype=np.float64)
    ham_r = np.array(hv, dtype=np.complex128).reshape(-1, 1, 1)
    return rvec, ham_r


def two_orbital_hoppings(t1=1.0, t2=0.5, de=0.4, V=0.2):
    """Two-orbital square lattice: diagonal hoppings, crystal field, hybridization."""
    rvec = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]], dtype=np.float64)
    onsite = np.array([[0.0, V], [V, de]], dtype=np.complex128)
    hop = np.diag([-t1, -t2]).astype(np.complex128)
    ham_r = np.array([onsite, hop, hop, hop, hop], dtype=np.complex128)
    return rvec, ham_r


def random_hoppings(Norb, seed, shells=((1, 0, 0), (1, 1, 0), (2, 0, 0)), sigma=0.3,
                    decay=0.4, onsite=0.3, bandwidth=None, complex_hop=False, dim=2):
    """Seeded multi-orbital model with H(-R) = H(R)^dagger (Hermitian H(k)).

    Shells are lattice vectors whose point-group images are all included; the
    hopping amplitude of shell s is N(0, sigma) * decay**s.  With
    ``complex_hop=False`` H(R) is real and symmetric, so the model also has
    inversion (H(-R) = H(R)) and the irreducible-k TRS reduction is exact."""
    rng = np.random.default_rng(seed)
    vecs = {(0, 0, 0): None}
    for s, base in enumerate(shells):
        b = np.array(base)
        imgs = set()
        for perm in ((0, 1, 2), (1, 0, 2)) if dim == 2 else ((0, 1, 2), (1, 0, 2), (2, 1, 0), (0, 2, 1), (1, 2, 0), (2, 0, 1)):
            for sx in (1, -1):
                for sy in (1, -1):
                    for sz in (1, -1):
                        v = b[list(perm)] * np.array([sx, sy, sz])
                        if dim == 2 and v[2] != 0:
                            continue
                        imgs.add(tuple(int(x) for x in v))
        for v in sorted(imgs):
            vecs.setdefault(v, s)
    rlist = sorted(vecs.keys())
    Nr = len(rlist)
    H = np.zeros((Nr, Norb, Norb), dtype=np.complex128)
    idx = {r: i for i, r in enumerate(rlist)}
    done = set()
    for r in rlist:
        if r in done:
            continue
        mr = tuple(-x for x in r)
        if r == (0, 0, 0):
            A = rng.normal(0.0, 0.1, (Norb, Norb))
            A = 0.5 * (A + A.T)
            A[np.diag_indices(Norb)] = rng.uniform(-onsite, onsite, Norb)
            H[idx[r]] = A
            done.add(r)
            continue
        s = vecs[r]
        amp = sigma * decay ** s
        A = rng.normal(0.0, amp, (Norb, Norb))
        if complex_hop:
            A = A + 1j * rng.normal(0.0, amp, (Norb, Norb))
            H[idx[r]] = A
            H[idx[mr]] = np.conj(A.T)
        else:
            A = 0.5 * (A + A.T)
            H[idx[r]] = A
            H[idx[mr]] = A
        done.add(r)
        done.add(mr)
    rvec = np.array(rlist, dtype=np.float64)
    # ham_r in the Python layout: ham_r[j, l, m] = Fortran ham_r(m, l, j)
    ham_r = np.ascontiguousarray(np.transpose(H, (0, 2, 1)))
    if bandwidth is not None:
        k = np.stack(np.meshgrid(np.arange(16) / 16, np.arange(16) / 16, indexing="ij"), -1).reshape(-1, 2)
        k = np.concatenate([k, np.zeros((len(k), 1))], axis=1)
        ph = np.exp(-2j * PI * k @ rvec.T)
        Hk = np.einsum("kr,rml->kml", ph, H)
        e = np.linalg.eigvalsh(0.5 * (Hk + np.conj(np.swapaxes(Hk, 1, 2))))
        ham_r = ham_r * (bandwidth / (e.max() - e.min()))
    return rvec, ham_r


def spin_orbit_hoppings(rvec, ham_r, alpha=0.0):
    """Spin-orbital model of a spatial model: spin-up orbitals first, then
    their spin-down partners (the default slist / invs of pyrpa's main.py),
    plus a Rashba term alpha (sin ky s_x - sin kx s_y).  Returns
    (rvec, ham_r, slist, invs) with invs 1-based.  The Rashba term keeps
    time reversal, H(-k)_ab = s_a s_b H(k)_{b'a'}, which the reference's
    irreducible-k scheme needs."""
    n = ham_r.shape[1]
    H = np.zeros((len(rvec), 2 * n, 2 * n), dtype=np.complex128)
    H[:, :n, :n] = ham_r
    H[:, n:, n:] = ham_r
    if alpha:
        sx = np.array([[0, 1], [1, 0]], dtype=np.complex128)
        sy = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
        for r, R in enumerate(np.asarray(rvec)):
            for d, Mspin, sgn in ((0, sy, -1.0), (1, sx, 1.0)):
                e = np.zeros(3)
                e[d] = 1.0
                if np.allclose(R, e):
                    c = 0.5j
                elif np.allclose(R, -e):
                    c = -0.5j
                else:
                    continue
                H[r] += np.kron(Mspin, np.eye(n)) * (alpha * sgn * c)
    slist = np.array([1] * n + [-1] * n, dtype=np.int64)
    invs = np.concatenate([np.arange(n, 2 * n), np.arange(n)]).astype(np.int64) + 1
    return rvec, H, slist, invs


def full_grid_dispersion_1orb(ham_r, rvec, Nx, Ny, Nz=1):
    """One-orbital band energy on the full grid [Nx,Ny,Nz]."""
    ix, iy, iz = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    k = np.stack([ix.ravel() / Nx, iy.ravel() / Ny, iz.ravel() / Nz], axis=1)
    e = (np.exp(-2j * PI * k @ rvec.T) @ ham_r[:, 0, 0]).real
    return e.reshape(Nx, Ny, Nz)


def two_pole(eps, a, delta):
    """Poles E and weights W of G = 1/(x - eps - a^2/(x - delta))."""
    eps = np.asarray(eps, dtype=np.float64)
    if a == 0.0:
        return np.stack([eps, eps]), np.full((2,) + eps.shape, 0.5)
    tr = eps + delta
    det = eps * delta - a * a
    disc = np.sqrt(np.maximum(tr * tr - 4.0 * det, 1e-300))
    Ep, Em = 0.5 * (tr + disc), 0.5 * (tr - disc)
    return np.stack([Ep, Em]), np.stack([(Ep - delta) / (Ep - Em), (Em - delta) / (Em - Ep)])


def two_pole_green(eig, temp, mu, Nw, a=0.0, delta=0.0):
    """[1,1,Nw,Nk] Green function with the two-pole self-energy (a=0: free)."""
    x = mu + 1j * (2 * np.arange(Nw) + 1) * PI * temp
    e = np.asarray(eig)[:, 0]
    sig = a * a / (x - delta) if a != 0.0 else 0.0
    G = 1.0 / (x[None, :] - e[:, None] - (sig[None, :] if a != 0.0 else 0.0))
    return np.ascontiguousarray(G.T[None, None])


def exact_chi0_1orb(eps_full, qlist, mlist, temp, mu, a=0.0, delta=0.0):
    """Exact bubble chi(q, i nu_m) = -T/N sum G(k+q, iw+inu) G(k, iw)."""
    Nx, Ny, Nz = eps_full.shape
    E, W = two_pole(eps_full, a, delta)
    out = np.zeros((len(qlist), len(mlist)), dtype=complex)
    for iq, q in enumerate(qlist):
        sh = tuple(-int(round(q[d] * n)) % n for d, n in enumerate((Nx, Ny, Nz)))
        Eq = np.roll(E, sh, axis=(1, 2, 3))
        Wq = np.roll(W, sh, axis=(1, 2, 3))
        for jm, m in enumerate(mlist):
            nu = 2 * PI * m * temp
            tot = 0.0j
            for p in range(2):
                for pp in range(2):
                    fa, fb = fermi(Eq[p], temp, mu), fermi(E[pp], temp, mu)
                    de = 1j * nu + E[pp] - Eq[p]
                    deg = (m == 0) & (np.abs(Eq[p] - E[pp]) < 1e-9)
                    safe = np.where(np.abs(de) < 1e-30, 1.0, de)
                    tot += (Wq[p] * W[pp] * np.where(deg, fb * (1 - fb) / temp, (fa - fb) / safe)).sum()
            out[iq, jm] = tot / (Nx * Ny * Nz)
    return out


def fit_power_order(ns, errs):
    return -np.polyfit(np.log(np.asarray(ns, float)), np.log(np.asarray(errs, float)), 1)[0]
