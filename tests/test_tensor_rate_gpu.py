"""Measured rates of the tensor instructions the residue GEMM could be built on
(sdpg_probe_tensor_rate): tcgen05.mma kind::f16, the legacy mma.sync with 8-bit integer
operands (tcgen05.mma kind::i8 does not exist for sm_103a; test_tensor_kinds_cpu.py), and
mma.sync with fp16 operands.  Each rate is printed; the test asserts only that each
probe ran and that the tcgen05 product is the fastest of the three."""
import pytest


@pytest.mark.gpu
def test_tensor_instruction_rates(sdpg):
    rates = {k: sdpg.probe_tensor_rate(k) for k in sdpg.TENSOR_PROBE_KINDS}
    for k, r in rates.items():
        print(f"\n{sdpg.TENSOR_PROBE_KINDS[k]}: {r / 1e12:.1f} T ops/s")
        assert r > 1e12, (k, r)
    assert rates[0] > rates[1] and rates[0] > rates[2], rates
    assert sdpg.tensor_error(0) == 0
