"""The exact and fused FP32 Black-Scholes kernels price two options at a time on
Blackwell's packed FP32 instructions (nt2cuda/bs_x2.cuh).  Their two-lane exp,
log, erfc and normcdf (and the table expressions' two-lane pow) must give the
one-lane functors' bits for every float argument, in NT2's twice-rounded arithmetic and with each fma/fnms one hardware
FMA (the fused mode): each check below runs over all 2^32 bit patterns on the
GPU and must find no difference (NaN-ness must agree; payloads are not
compared)."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("which,name", [(0, "exp"), (1, "log"), (2, "erfc(|a|)"), (3, "normcdf(a), normcdf(-a)")])
def test_two_lane_functor_is_bit_exact_over_every_float(gpu, cuda_lib, which, name, fused):
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(which + (4 if fused else 0), C.byref(n), first,
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (name, n.value, [hex(first[i]) for i in range(min(8, n.value))])


@pytest.mark.parametrize("which,name", [(8, "exp_small"), (9, "log"), (10, "erfc(|a|), Numerical Recipes fit"),
                                        (11, "normcdf(a), normcdf(-a)")])
def test_two_lane_fast_functor_matches_one_lane_over_every_float(gpu, cuda_lib, which, name):
    """The fast precision mode's packed functors give its one-lane functors' bits
    (ex2/lg2/reciprocals per lane, the FMAs, multiplies and adds packed)."""
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(which, C.byref(n), first, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (name, n.value, [hex(first[i]) for i in range(min(8, n.value))])


@pytest.mark.parametrize("fused", [False, True])
def test_two_lane_fastnormcdf_is_bit_exact_over_every_float(gpu, cuda_lib, fused):
    """The demo form's cdf (fastnormcdf, Abramowitz-Stegun 26.2.17) packed two lanes
    per instruction gives the one-lane functor's bits, unfused and fused."""
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(13 if fused else 12, C.byref(n), first,
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (n.value, [hex(first[i]) for i in range(min(8, n.value))])


@pytest.mark.parametrize("which,name", [(14, "sin"), (15, "cos"), (16, "sin, fused"), (17, "cos, fused"),
                                        (18, "tan"), (19, "cot"), (20, "tan, fused"), (21, "cot, fused")])
def test_two_lane_sine_cosine_evaluation_over_every_float(gpu, cuda_lib, which, name):
    """The float trigonometric functors evaluate their polynomials (sine and cosine,
    or tangent) two lanes per packed instruction; over every reduced argument (and each
    quadrant and sign) the result is the one-lane evaluation's."""
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(which, C.byref(n), first, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (name, n.value, [hex(first[i]) for i in range(min(8, n.value))])


@pytest.mark.parametrize("which,name", [(22, "pow"), (23, "pow, fused"), (24, "pow_abs"), (25, "pow_abs, fused")])
def test_two_lane_pow_matches_one_lane(gpu, cuda_lib, which, name):
    """FP32 pow and pow_abs run two lanes per packed instruction (the division of
    the reduced mantissa by its table value through a reciprocal, a Newton step and
    Markstein's correction); every float is tried as the base and as the exponent,
    each against a drawn partner, and both lanes must give the one-lane bits."""
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(which, C.byref(n), first, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (name, n.value, [hex(first[i]) for i in range(min(8, n.value))])


@pytest.mark.parametrize("which,name", [(26, "cbrt"), (27, "cbrt, fused")])
def test_two_lane_cbrt_is_bit_exact_over_every_float(gpu, cuda_lib, which, name):
    """FP32 cbrt nodes run two lanes per packed instruction, the Newton step's division by a
    reciprocal, a Newton step and Markstein's correction where the residual stays exact; over
    every float both lanes give the one-lane bits."""
    n = C.c_ulonglong(99)
    first = (C.c_uint32 * 8)()
    st = cuda_lib.nt2cuda_selftest_x2(which, C.byref(n), first, torch.cuda.current_stream().cuda_stream)
    assert st == 0
    assert n.value == 0, (name, n.value, [hex(first[i]) for i in range(min(8, n.value))])
