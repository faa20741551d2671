"""Packed parameter sweep on the GPU: instances solved from several host
threads, each on its own engine context and CUDA stream, give the same
results as the one-after-another loop, and a failure in one thread's
context is reported to that thread only."""
import threading

import numpy as np
import pytest

from pyrpa_gb300 import sweep as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    from pyrpa_gb300 import build, flibs
    if not build.LIB.exists():
        build.build()
    flibs.load_library()
    flibs.set_verbose(0)
    return flibs


def _instances():
    # uneven small instances: 1-2 orbitals, 16^2 and 32^2 meshes, 256 and 512 frequencies
    shapes = [(1, 16, 256), (2, 16, 512), (1, 32, 256), (2, 32, 256), (1, 16, 512), (2, 16, 256)]
    return [S.Instance(index=i, Norb=o, N=n, Nw=w, seed=1000 + 7 * i, u_frac=0.6 + 0.05 * i,
                       temp=0.02 + 0.004 * i, n_per_orb=0.8 + 0.02 * i) for i, (o, n, w) in enumerate(shapes)]


@pytest.mark.parametrize("precision", [3264, 64])
def test_packed_sweep_equals_the_sequential_loop(F, precision):
    insts = _instances()
    seq = S.run(insts, eps=1e-6, precision=precision)
    packed = S.run_packed(insts, workers=3, eps=1e-6, precision=precision)
    F.set_precision(64)
    assert [r["index"] for r in packed] == [r["index"] for r in seq]
    for a, b in zip(seq, packed):
        assert "error" not in a and "error" not in b
        assert a["iterations"] == b["iterations"]
        assert a["mu"] == b["mu"] and a["esterr"] == b["esterr"] and a["stoner"] == b["stoner"]
        assert a["sigma_abs_sum"] == b["sigma_abs_sum"]


def test_errors_stay_in_their_thread(F):
    """A singular (I - chi0 S) in one thread's context while another thread
    solves a regular model: only the first call fails."""
    import _models as M
    from oracle import api as O
    rvec, ham_r = M.square_hoppings(1.0, 0.5)
    klist, kmap, invk = O.gen_irr_k_TRS(8, 8, 1)
    hamk = O.gen_ham(klist, ham_r, rvec)
    eig, uni = O.get_eig(hamk)
    olist, site = O.get_chi_orb_list(1)
    olist = np.asfortranarray(olist)
    S1, C1 = O.gen_SCmatrix(olist, site, 2.0, 0.0)
    chi = 0.05 * np.ones((1, 1, 4, 3), dtype=np.complex128)
    chi[0, 0, 0, 0] = 1.0 / S1[0, 0]
    out = {}
    barrier = threading.Barrier(2)

    def singular():
        F.set_thread_stream(True)
        try:
            barrier.wait()
            for _ in range(20):
                try:
                    F.get_Vsigma_nosoc_flex(chi, S1, C1)
                    out.setdefault("singular", "no error")
                except RuntimeError as e:
                    out.setdefault("singular", str(e))
        finally:
            F.set_thread_stream(False)

    def regular():
        F.set_thread_stream(True)
        try:
            F.set_precision(64)
            barrier.wait()
            res = []
            for _ in range(5):
                sg, mu = F.mkself(S1 * 0.5, C1 * 0.5, kmap, invk, olist, hamk, eig, uni, 0.0, 0.4, 0.1, 16, 8, 8, 1,
                                  False, False, eps=1e-8, pp=0.5)
                res.append((mu, float(np.abs(sg).sum()), F.last_error()))
            out["regular"] = res
        except Exception as e:  # noqa: BLE001
            out["regular"] = repr(e)
        finally:
            F.set_thread_stream(False)

    ts = [threading.Thread(target=singular), threading.Thread(target=regular)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert "zgesv failed" in out["singular"]
    assert isinstance(out["regular"], list), out["regular"]
    assert all(e == "" for _, _, e in out["regular"])
    assert len({(m, s) for m, s, _ in out["regular"]}) == 1
    F.set_precision(64)
    sg, mu = F.mkself(S1 * 0.5, C1 * 0.5, kmap, invk, olist, hamk, eig, uni, 0.0, 0.4, 0.1, 16, 8, 8, 1, False,
                      False, eps=1e-8, pp=0.5)
    assert (mu, float(np.abs(sg).sum())) == out["regular"][0][:2]
