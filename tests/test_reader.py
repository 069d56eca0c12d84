"""Host-side problem and parameter readers (IO::read, Parameter::readFile) and
the synthetic generators' determinism (the GPU machine regenerates the golden
inputs and must get byte-identical files)."""
import hashlib
import json
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_param_read(sdpg):
    p = sdpg.Param.read(os.path.join(GOLDEN, "example1.param"))
    assert (p.maxIteration, p.precision) == (200, 200)
    assert p.epsilonStar == 1.0e-30 and p.lambdaStar == 1.0e4 and p.gammaStar == 0.9
    d = sdpg.Param.default(1)
    assert (d.maxIteration, d.precision, d.gammaStar) == (1000, 300, 0.5)


def test_read_example1(sdpg):
    pr = sdpg.Problem.read(os.path.join(GOLDEN, "example1.dat-s"))
    assert pr.h


def test_read_errors(sdpg, tmp_path):
    with pytest.raises(sdpg.SdpgError):
        sdpg.Problem.read(str(tmp_path / "missing.dat-s"))
    bad = tmp_path / "bad.dat-s"
    bad.write_text('"t"\n2 = m\n1\n2\n1 1\n1 1 3 1 1.0\n')
    with pytest.raises(sdpg.SdpgError):
        sdpg.Problem.read(str(bad))


@pytest.mark.parametrize("name", ["maxcut20", "maxcut40", "control20", "control30", "gpp40", "gpp60",
                                  "maxcut100", "maxcut124pm"])
def test_generators_reproduce_golden_inputs(problems, name):
    g = json.load(open(os.path.join(GOLDEN, name + ".json")))
    kw = {k: (tuple(v) if isinstance(v, list) else v) for k, v in g["kwargs"].items()}
    text = getattr(problems, g["generator"])(**kw).text()
    assert hashlib.sha256(text.encode()).hexdigest() == g["sha256"]


def test_programmatic_problem(sdpg):
    pr = sdpg.Problem.new(3, [2])
    for k, v in enumerate(["48", "-8", "20"], start=1):
        pr.set_c(k, v)
    for e in [(0, 1, 1, 1, "-11"), (0, 1, 2, 2, "23"), (1, 1, 1, 1, "10"), (1, 1, 1, 2, "4"), (2, 1, 2, 2, "-8"),
              (3, 1, 1, 2, "-8"), (3, 1, 2, 2, "-2")]:
        pr.add_entry(*e)
    with pytest.raises(sdpg.SdpgError):
        pr.add_entry(1, 1, 3, 1, "1")
