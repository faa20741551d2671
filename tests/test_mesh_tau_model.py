"""Index model of the mesh-by-time kernels (csrc/flex.cu: mesh_tau_grid and
mesh_tau), on CPU.

Kernels over a padded array of P = Nkall x M points (the pads, the chi0
product and scatter, the tau reference, the Sigma contraction, the output
scatters) launch mesh_tau_grid(Nkall, M, ny, chunk) blocks of 256 threads;
a thread maps its block and lane to one mesh point r and the slices
t0 <= t < t1 of a chunk.  This test restates that mapping in numpy and
checks that every point (r, t) of the array is visited exactly once, by a
thread with r < Nkall, for mesh and time sizes of the benchmark and sweep
models and ragged edges, so that no element is lost or written twice."""
import numpy as np
import pytest

THREADS = 256
CHUNK = 8


def grid(nkall, m, chunk=CHUNK):
    nrb = (nkall + THREADS - 1) // THREADS
    nch = (m + chunk - 1) // chunk
    return nrb * nch


def visits(nkall, m, chunk=CHUNK):
    nblocks = grid(nkall, m, chunk)
    nrb = (nkall + THREADS - 1) // THREADS
    b = np.arange(nblocks)[:, None]
    lane = np.arange(THREADS)[None, :]
    rb, tc = b % nrb, b // nrb
    r = (rb * THREADS + lane).ravel()
    t0 = np.broadcast_to(tc * chunk, (nblocks, THREADS)).ravel()
    t1 = np.minimum(m, t0 + chunk)
    keep = r < nkall
    count = np.zeros((m, nkall), dtype=np.int64)
    for rr, a, z in zip(r[keep], t0[keep], t1[keep]):
        count[a:z, rr] += 1
    return count


@pytest.mark.parametrize("nkall,m,chunk", [
    (64 * 64, 64, CHUNK),       # c2 mesh, a short time axis (the full 4096 is the same pattern)
    (32 * 32, 2048, CHUNK),     # c1 mesh and time axis
    (24 ** 3, 16, CHUNK),       # c5 mesh (not a multiple of 256)
    (16, 32, CHUNK),            # a 4 x 4 test mesh: most lanes idle
    (6 ** 3, 20, CHUNK),        # ragged time chunk
    (2050, 1024, CHUNK),        # irreducible k x frequencies (the scatters)
    (64 * 64, 20, 1),           # one slice per thread (the Sigma contraction)
])
def test_every_point_once(nkall, m, chunk):
    c = visits(nkall, m, chunk)
    assert c.shape == (m, nkall)
    assert (c == 1).all()


def test_grid_fits_the_launch_limits():
    # the largest sweep array: 128 x 128 mesh, 8192 time slices, one slice per thread
    assert grid(128 * 128, 8192, 1) < 2 ** 31 - 1
    assert grid(128 * 128, 8192) * THREADS >= 128 * 128 * 8192 // CHUNK
