"""The split-BF16 tensor-core form of the line transforms, emulated on the
host (oracle/split_bf16_study.py): every DFT stage as BF16 matrix products with
exact products and FP32 sums, inside the multislice slice loop, against the
same loop in float64.  The 3-term split leaves an order of magnitude more
exit-wave error than FP32 stages (above the 1e-5 at which the tensor-core form
may be kept); the 6-term split is as accurate as FP32 but needs six tensor
products per stage.  No GPU."""
from oracle import split_bf16_study as sbs


def test_bf16_split_emulation_orders_the_forms(oracle):
    e = sbs.study(oracle, n=64, fov=32.0, natom=150)
    assert e["fp32"] < 1e-6
    assert e["3"] > 5.0 * e["fp32"]          # 16-bit products: far above FP32 rounding
    assert e["6"] < 2.0 * e["fp32"]          # 24-bit products: FP32-level


def test_bf16_rounding():
    import numpy as np
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 1e-30], np.float32)
    y = sbs.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0          # tie to even
    assert y[2] == np.float32(1.0078125)       # above the tie: rounds up
    assert abs(y[3] - x[3]) <= abs(x[3]) * 2.0 ** -8
    hi, lo = sbs.split(x[3:4], 2)
    assert abs((hi + lo)[0] - x[3]) <= abs(x[3]) * 2.0 ** -16
