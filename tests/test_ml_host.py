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
    assert s.startswith("3.14159265358979323846264338328")  # 30 digits, rounded half up
    assert sdpg.ml_to_double(sdpg.ml_from_double([1.5, -2.0**-300, 0.0], 8)).tolist() == [1.5, -2.0**-300, 0.0]


def test_precision_mapping(sdpg):
    assert sdpg.limbs_for_precision(200) == 8
    assert sdpg.limbs_for_precision(256) == 8
    assert sdpg.limbs_for_precision(512) == 16
    with pytest.raises(sdpg.SdpgError):
        sdpg.limbs_for_precision(1024)


def _py_format(x: Fraction, spec: str) -> str:
    """C printf semantics of one conversion with half-up rounding, via decimal
    (Python writes at least one exponent digit where C writes two: widened here)."""
    import decimal
    import re
    m = re.fullmatch(r"([<+]*)(\d*)\.(\d+)([eEf])", spec)
    flags, width, prec, conv = m.group(1), int(m.group(2) or 0), m.group(3), m.group(4)
    with decimal.localcontext() as ctx:
        ctx.prec = 400
        ctx.rounding = decimal.ROUND_HALF_UP
        d = decimal.Decimal(x.numerator) / decimal.Decimal(x.denominator)
        body = format(d, ("+" if "+" in flags else "") + "." + prec + conv)
    body = re.sub(r"([eE])([+-])(\d)$", r"\g<1>\g<2>0\g<3>", body)
    return body.ljust(width) if "<" in flags else body.rjust(width)


@pytest.mark.parametrize("limbs", [8, 16])
def test_gmp_printf_formats(sdpg, exact, limbs):
    """sdpg_ml_format_gmp against Python's decimal formatting (exact value, half-up
    rounding) for the conversions the result file uses and a few others."""
    rng = random.Random(77 + limbs)
    vals = exact.random_ml(60, limbs, rng, -200, 200)
    vals[0] = 0
    extra = sdpg.ml_parse(["5.9", "-1.375", "0.00449999", "9.9999999", "-0.5", "123456789.125", "1e-31"], limbs)
    vals = np.concatenate([vals, extra])
    fr = [exact.to_fraction(v) for v in exact.ml_decode(vals)]
    for fmt, spec in [("%+50.40Fe", "+50.40e"), ("%+8.3Fe", "+8.3e"), ("%10.16Fe", "10.16e"), ("%4.16Fe", "4.16e"),
                      ("%.6Fe", ".6e"), ("%-20.5FE", "<20.5E"), ("%.3Ff", ".3f"), ("%+12.0Ff", "+12.0f")]:
        got = sdpg.ml_format_gmp(vals, fmt)
        for g, x in zip(got, fr):
            if spec.endswith("f") and abs(x) > 10 ** 30:
                continue  # fixed notation of huge values: not used by result files
            # zero through C's own printf (Python's % operator on a float)
            want = (fmt.replace("F", "") % 0.0) if x == 0 else _py_format(x, spec)
            assert g == want, (fmt, g, want)
    # text around the conversion is copied
    assert sdpg.ml_format_gmp(extra[:1], "x=%+.2Fe;")[0] == "x=+5.90e+00;"
