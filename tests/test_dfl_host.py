"""Host build of the engine's double-float and complex helpers
(csrc/common.cuh: the double-word sum, product, fused multiply-add, Dekker
division, the complex reciprocal and division), checked on CPU against
long double.  The same inline functions run in the kernels (they are
__host__ __device__), so this pins their error bounds without a GPU: the
double-float arithmetic must stay within a few 2^-47 of the operands'
magnitudes, and the reciprocal within a few units in the last place of its
type."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = r'''
#include "common.cuh"
#include <cstdio>
#include <random>
using namespace pgb;
static long double ld(dfl a) { return (long double)a.hi + (long double)a.lo; }
static dfl mk(long double x) { const float h = (float)x; return dfl(h, (float)(x - (long double)h)); }
int main() {
  std::mt19937_64 rng(7);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_real_distribution<double> ue(-4.0, 4.0);
  auto draw = [&]() { return (long double)nd(rng) * expl((long double)ue(rng)); };
  long double e_add = 0, e_mul = 0, e_mad = 0, e_div = 0, e_rcp32 = 0, e_rcp64 = 0, e_rcpdf = 0, e_cmul = 0;
  for (int i = 0; i < 200000; ++i) {
    const long double x = draw(), y = draw(), z = draw();
    const dfl a = mk(x), b = mk(y), c = mk(z);
    const long double ax = ld(a), by = ld(b), cz = ld(c);
    e_add = fmaxl(e_add, fabsl(ld(a + b) - (ax + by)) / (fabsl(ax) + fabsl(by)));
    e_mul = fmaxl(e_mul, fabsl(ld(a * b) - ax * by) / fabsl(ax * by));
    e_mad = fmaxl(e_mad, fabsl(ld(mad(a, b, c)) - (ax * by + cz)) / (fabsl(ax * by) + fabsl(cz)));
    e_div = fmaxl(e_div, fabsl(ld(a / b) - ax / by) / fabsl(ax / by));
    // complex reciprocals: |1/b - exact| / |1/b|
    const long double u = draw(), v = draw(), m2 = u * u + v * v;
    const long double rx = u / m2, ry = -v / m2, rn = sqrtl(rx * rx + ry * ry);
    const float2 r32 = crecip(make_float2((float)u, (float)v));
    const long double u32 = (float)u, v32 = (float)v, m32 = u32 * u32 + v32 * v32;
    e_rcp32 = fmaxl(e_rcp32, hypotl(r32.x - u32 / m32, r32.y + v32 / m32) / sqrtl(1 / m32));
    const double2 r64 = crecip(make_double2((double)u, (double)v));
    const long double u64 = (double)u, v64 = (double)v, m64 = u64 * u64 + v64 * v64;
    e_rcp64 = fmaxl(e_rcp64, hypotl(r64.x - u64 / m64, r64.y + v64 / m64) / sqrtl(1 / m64));
    cdf bd;
    bd.x = mk(u);
    bd.y = mk(v);
    // complex product, normwise: |ab - exact| / (|a| |b|)
    cdf ad;
    ad.x = a;
    ad.y = b;
    const cdf pr = ad * bd;
    const long double px = ax * ld(bd.x) - by * ld(bd.y), py = ax * ld(bd.y) + by * ld(bd.x);
    e_cmul = fmaxl(e_cmul, hypotl(ld(pr.x) - px, ld(pr.y) - py) /
                               (hypotl(ax, by) * hypotl(ld(bd.x), ld(bd.y))));
    const cdf rd = crecip(bd);
    e_rcpdf = fmaxl(e_rcpdf, hypotl(ld(rd.x) - rx, ld(rd.y) - ry) / rn);
  }
  printf("%Le %Le %Le %Le %Le %Le %Le %Le\n", e_add, e_mul, e_mad, e_div, e_rcp32, e_rcp64, e_rcpdf, e_cmul);
  return 0;
}
'''


@pytest.fixture(scope="module")
def errors(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("dfl")
    (d / "t.cu").write_text(SRC)
    exe = d / "t"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(ROOT / "pyrpa_gb300" / "csrc"), str(d / "t.cu"), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    return dict(zip(["add", "mul", "mad", "div", "rcp32", "rcp64", "rcpdf", "cmul"], map(float, out)))


def test_double_float_sum_product_mad_division(errors):
    u = 2.0 ** -48
    # measured on this draw: add 2.3 u, mul 3.4 u, mad 4.3 u, div 6.7 u
    assert errors["add"] < 4 * u       # normwise, Dekker's add2
    assert errors["mul"] < 6 * u
    assert errors["mad"] < 8 * u       # one renormalization for the product and the sum
    assert errors["div"] < 12 * u
    assert errors["cmul"] < 8 * u      # complex product: one sum of two double-word products a component


def test_complex_reciprocals(errors):
    # measured: 2.9 ulp (FP32), 2.9 ulp (FP64), 5 u (double-float)
    assert errors["rcp32"] < 4 * 2.0 ** -24
    assert errors["rcp64"] < 4 * 2.0 ** -53
    assert errors["rcpdf"] < 16 * 2.0 ** -48
