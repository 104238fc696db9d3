"""The boundary network's CPU oracle: its backward pass against central differences (float64,
rounding off), its BF16 rounding against known values, and the parameter layout."""
import numpy as np

from oracle import mlp_oracle as M


def test_backward_matches_central_differences():
    assert M.fd_check(seed=3) < 1e-6


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.1415927, 0.0], np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1.0; 1.005859375 rounds up
    assert list(M.bf16(x)) == [1.0, 1.0, 1.0078125, -2.5, 3.140625, 0.0]


def test_layout():
    assert M.N_PARAMS == 64 * 81 + 64 + 64 * 64 + 64 + 64 + 1
    p = np.arange(M.N_PARAMS, dtype=np.float64)
    assert np.array_equal(M.pack(M.unpack(p)), p)
