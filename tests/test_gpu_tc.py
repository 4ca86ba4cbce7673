"""Tensor-core GEMMs (tcgen05, used by the mixed-precision CCD) against FP64.

Error scale of a hi/lo split product: BF16 pairs carry ~16 significant bits, TF32
pairs ~22, but both accumulate in FP32 tensor memory, which bounds the relative error
near 1e-5 for K ~ 1500 either way; dropping the A_lo term leaves the 8-bit BF16
rounding of A (~2e-3)."""
import pytest

pytestmark = pytest.mark.gpu

SMALL = [(128, 16, 64)]
RAGGED = [(300, 80, 700), (129, 17, 65), (1000, 256, 1500), (64, 48, 40), (777, 66, 1392)]


@pytest.mark.parametrize("shapes", [SMALL, RAGGED], ids=["single_tile", "ragged_grouped"])
def test_bf16x3_matches_fp64(ccx, shapes):
    err, ms = ccx.selftest_tc_gemm(shapes, kind=0, use_alo=True)
    assert err < 2e-4, err


def test_tf32x3_matches_fp64(ccx):
    err, ms = ccx.selftest_tc_gemm(RAGGED, kind=1, use_alo=True)
    assert err < 5e-5, err
    err1, _ = ccx.selftest_tc_gemm(SMALL, kind=1, use_alo=True)
    assert err1 < 2e-6, err1  # short K: the TF32 split itself, ~1e-6


def test_dropping_a_lo_is_less_accurate(ccx):
    full, _ = ccx.selftest_tc_gemm(RAGGED, kind=0, use_alo=True)
    two, _ = ccx.selftest_tc_gemm(RAGGED, kind=0, use_alo=False)
    assert two > 10 * full and two < 2e-2


@pytest.mark.parametrize("shapes", [SMALL, RAGGED], ids=["single_tile", "ragged_grouped"])
def test_ozaki_digit_gemm_is_fp64_accurate(ccx, shapes):
    """kind 2: 9 six-bit digits per operand, exact FP32 level sums; against a long
    double reference the error stays at the FP64 rounding level (FP64 GEMM itself is
    ~sqrt(K) 2^-53 relative to sum |a||b|, here ~1e-14 of max |AB|)."""
    err, ms = ccx.selftest_tc_gemm(shapes, kind=2)
    assert err < 1e-13, err


WIDE = [(200, 300, 150), (129, 520, 700), (300, 16, 90)]


@pytest.mark.parametrize("kind", [0, 2], ids=["bf16x3", "digits"])
def test_wide_n_column_blocks(ccx, kind):
    """N beyond one 256-column accumulator: column blocks that step through the whole B."""
    err, _ = ccx.selftest_tc_gemm(WIDE, kind=kind)
    assert err < (2e-4 if kind == 0 else 1e-13), err


@pytest.mark.parametrize("kind", [0, 1], ids=["bf16x3", "tf32x3"])
def test_segmented_products_one_accumulator(ccx, kind):
    """Several products (K cut into separately tiled segments) accumulated into one tile and
    written once with a C0 term, overwriting C or adding to it; wide N in column blocks."""
    shapes = RAGGED + WIDE
    err, _ = ccx.selftest_tc_gemm(shapes, kind=kind, segments=True)
    assert err < (2e-4 if kind == 0 else 5e-5), err
