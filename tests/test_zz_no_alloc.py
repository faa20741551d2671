"""The allocation-free entry point pyrpa_gb_eig_or_tr_chi_noalloc against
the allocating get_eig_or_tr_chi, through the C ABI, on two calls in a row.

Collected last: its device buffers come from torch, which the test uses only
to hold device memory; the entry point itself allocates none."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry():
    torch = pytest.importorskip("torch")
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    F.set_verbose(0)
    klist, kmap, invk = F.gen_irr_k_TRS(8, 8, 1)
    Nk, Nkall = len(klist), len(invk)
    rng = np.random.default_rng(17)
    d_invk = torch.from_numpy(np.ascontiguousarray(invk)).cuda()
    stream = torch.cuda.current_stream()
    for Nchi in (4, 9):
        for sw in (True, False):
            for call in range(2):  # two calls in a row, different inputs
                chi = rng.standard_normal((Nchi, Nchi, Nk)) + 1j * rng.standard_normal((Nchi, Nchi, Nk))
                chi = np.ascontiguousarray(chi)
                ref = F.get_eig_or_tr_chi(chi, invk, sw)
                d_chi = torch.from_numpy(chi).cuda()
                d_out = torch.full((Nkall,), float("nan"), dtype=torch.complex128, device="cuda")
                torch.cuda.synchronize()
                F.eig_or_tr_chi_noalloc(d_out.data_ptr(), d_chi.data_ptr(), d_invk.data_ptr(), Nkall, Nk, Nchi, sw,
                                        stream.cuda_stream)
                stream.synchronize()
                got = d_out.cpu().numpy()
                assert np.array_equal(got, ref), (Nchi, sw, call, np.abs(got - ref).max())


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    from pyrpa_gb300 import flibs as F
    F.load_library()
    with pytest.raises(RuntimeError, match="65536"):
        # rejected on the host before any launch; the pointers are never used
        F.eig_or_tr_chi_noalloc(16, 16, 16, 200000, 100001, 4, True, 0)
