"""Host-side multi-limb arithmetic (the scalar engine shared by kernels and the
IPM control logic) against exact rational arithmetic from the oracle."""
import random
from fractions import Fraction

import numpy as np
import pytest


@pytest.mark.parametrize("limbs", [8, 16])
def test_add_sub_mul_div_sqrt(sdpg, exact, limbs):
    rng = random.Random(1234 + limbs)
    n = 300
    a = exact.random_ml(n, limbs, rng, -40, 40)
    b = exact.random_ml(n, limbs, rng, -40, 40)
    # include near-cancellation pairs and exact zeros
    b[:20] = a[:20]
    b[20:40, 1] ^= 1
    b[20:40] = a[20:40].copy()
    b[20:40, 1] ^= 1
    a[40:45] = 0
    ea, eb = exact.ml_decode(a), exact.ml_decode(b)
    ulp = Fraction(1, 1 << (32 * limbs - 3))  # a few units in the last place
    for op, f in [(sdpg.OP_ADD, lambda x, y: x + y), (sdpg.OP_SUB, lambda x, y: x - y),
                  (sdpg.OP_MUL, lambda x, y: x * y)]:
        got = exact.ml_decode(sdpg.ml_host_op(op, a, b))
        for i in range(n):
            x, y = exact.to_fraction(ea[i]), exact.to_fraction(eb[i])
            ref = f(x, y)
            err = abs(exact.to_fraction(got[i]) - ref)
            scale = max(abs(x), abs(y)) if op != sdpg.OP_MUL else abs(ref)
            assert err <= ulp * scale, (op, i)
    nz = np.array([i for i in range(n) if eb[i][0] != 0])
    got = exact.ml_decode(sdpg.ml_host_op(sdpg.OP_DIV, a[nz], b[nz]))
    for k, i in enumerate(nz):
        ref = exact.to_fraction(ea[i]) / exact.to_fraction(eb[i])
        assert abs(exact.to_fraction(got[k]) - ref) <= ulp * abs(ref)
    pos = a.copy()
    pos[:, 1] = 0
    got = exact.ml_decode(sdpg.ml_host_op(sdpg.OP_SQRT, pos))
    for i, (g, p) in enumerate(zip(got, exact.ml_decode(pos))):
        x = exact.to_fraction(p)
        r = exact.to_fraction(g)
        # |r^2 - x| <= 2 * r * err  ->  check r^2 against x
        assert abs(r * r - x) <= 4 * ulp * x, i


def test_parse_format_roundtrip(sdpg, exact):
    vals = ["1", "-11", "0.25", "-2.5e-3", "123456789.000000001", "1e-70", "7.0E4", "0"]
    arr = sdpg.ml_parse(vals, 8)
    dec = exact.ml_decode(arr)
    for t, d in zip(vals, dec):
        ref = Fraction(t.lower().replace("e", "e")) if "e" not in t.lower() else Fraction(t)
        got = exact.to_fraction(d)
        assert abs(got - ref) <= abs(ref) / (1 << 250)
    s = sdpg.ml_format(sdpg.ml_parse(["3.14159265358979323846264338327950288"], 8), 30)[0]
    assert s.startswith("3.14159265358979323846264338327")
    assert sdpg.ml_to_double(sdpg.ml_from_double([1.5, -2.0**-300, 0.0], 8)).tolist() == [1.5, -2.0**-300, 0.0]


def test_precision_mapping(sdpg):
    assert sdpg.limbs_for_precision(200) == 8
    assert sdpg.limbs_for_precision(256) == 8
    assert sdpg.limbs_for_precision(512) == 16
    with pytest.raises(sdpg.SdpgError):
        sdpg.limbs_for_precision(1024)
