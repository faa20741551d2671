"""The allocation-free entry point pyrpa_gb_eig_or_tr_chi_noalloc against
the allocating get_eig_or_tr_chi, through the C ABI, on two calls in a row.

The entry point is for callers that cannot let this library allocate device
memory: a framework whose caching allocator already holds most of HBM, or a
loop that enqueues on its own stream without a host round trip per call.
Its first call on a device does the one-time set-up (it takes what the
library's module needs on that device under lazy loading), so the test makes
that call before any other call into the library; the test then passes the
same way alone in a fresh process and after every other test.  It is
collected last (file name) so that a run stopping at its first failure has
run everything else.  Device buffers come from torch, used only to hold
device memory; the entry point itself allocates none.  Results must equal
the allocating entry's bit for bit: both run the same kernel on the same
data.  Sizes: Nchi = 4 and 9 on an 8x8 mesh, and Nchi = 25 (five orbitals,
the benchmark's vertex size) on the benchmark's 64x64 mesh.
"""
import numpy as np
import pytest

from oracle import api as O

pytestmark = pytest.mark.gpu


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_noalloc_matches_allocating_entry():
    torch = pytest.importorskip("torch")
    from pyrpa_gb300 import build, flibs as F
    if not build.LIB.exists():
        build.build()
    F.load_library()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(17)
    for N, Nchi in ((8, 4), (8, 9), (64, 25)):
        klist, _, invk = O.gen_irr_k_TRS(N, N, 1)
        Nkall, Nk = len(invk), len(klist)
        d_invk = _device(torch, invk)
        for sw in (True, False):
            outs = []
            for call in range(2):  # two calls in a row, different inputs
                chi = rng.standard_normal((Nchi, Nchi, Nk)) + 1j * rng.standard_normal((Nchi, Nchi, Nk))
                chi = np.ascontiguousarray(chi)
                d_chi = _device(torch, chi)
                d_out = torch.full((Nkall,), float("nan"), dtype=torch.complex128, device="cuda")
                torch.cuda.synchronize()
                F.eig_or_tr_chi_noalloc(d_out.data_ptr(), d_chi.data_ptr(), d_invk.data_ptr(), Nkall, Nk, Nchi, sw,
                                        stream.cuda_stream)
                stream.synchronize()
                got = d_out.cpu().numpy()
                # the allocating entry runs only after the first no-alloc call
                ref = F.get_eig_or_tr_chi(chi, invk, sw)
                assert np.array_equal(got, ref), (Nchi, sw, call, np.abs(got - ref).max())
                outs.append(got)
            assert not np.array_equal(outs[0], outs[1])


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    from pyrpa_gb300 import flibs as F
    F.load_library()
    with pytest.raises(RuntimeError, match="65536"):
        # rejected on the host before any launch; the pointers are never used
        F.eig_or_tr_chi_noalloc(16, 16, 16, 200000, 100001, 4, True, 0)
