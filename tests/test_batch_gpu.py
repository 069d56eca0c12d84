"""Batched solves (sdpg_solve_batch): many problems with several solvers in flight at
once must give exactly the results of solving each problem alone — the solvers share
nothing but the GPU, and every reduction runs in a fixed order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(problems_mod, sdpg):
    out = []
    for seed, (m, blocks) in enumerate([(20, (15, 16)), (26, (17, 15)), (31, (15, 18)), (23, (16, 16)),
                                       (35, (18, 15))]):
        rng = np.random.default_rng(1000 + seed)
        c, F0, F = problems_mod.control_dense(m, blocks, rng)
        out.append(sdpg.Problem.from_dense(c, F0, F))
    return out


def test_batch_matches_individual_solves(sdpg, problems):
    probs = _instances(problems, sdpg)
    param = sdpg.Param.default()
    ref_its, ref_info = [], []
    for p in probs:
        s = sdpg.Solver(p, param)
        ref_its.append(s.run())
        info = s.info()
        ref_info.append([sdpg.PHASES.index(info[k]) if k == "phase" else info[k] for k in sdpg.INFO_KEYS])
        s.close()
    its, info = sdpg.solve_batch(probs, param, concurrency=3)
    assert list(its) == ref_its
    assert np.array_equal(info, np.array(ref_info)), np.abs(info - np.array(ref_info)).max()
    # control-type instances are strictly feasible: every solve reaches pdOPT
    assert all(sdpg.PHASES[int(row[0])] == "pdOPT" for row in info)


def test_batch_member_without_constraints_does_not_disturb_others(sdpg, problems):
    """A member whose constraint matrices are all zero (its Schur matrix is singular,
    so its first Cholesky fails and the solve stops) leaves the others' results as they
    are when solved alone."""
    probs = _instances(problems, sdpg)[:2]
    bad = sdpg.Problem.new(3, [4])  # no constraint matrices: A_i = 0
    its, info = sdpg.solve_batch([probs[0], bad, probs[1]], concurrency=2)
    alone, info_alone = sdpg.solve_batch([probs[0], probs[1]], concurrency=1)
    assert its[0] == alone[0] and its[2] == alone[1]
    assert np.array_equal(info[[0, 2]], info_alone)
