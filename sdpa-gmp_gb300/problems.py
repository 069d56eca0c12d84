"""Seeded synthetic SDP generators, written in SDPA sparse format (``.dat-s``).

SDPA's ``.dat-s`` file describes ``F0..Fm`` and ``c``; the solver's internal
problem is ``min C.X  s.t. A_i.X = b_i, X >= 0`` with ``C = -F0``,
``A_i = F_i`` and ``b = c`` (reader: sdpa_io.cpp:626-663, the ``-value`` for
``k == 0`` at sdpa_io.cpp:661).  Every generator below therefore writes
``F0 = -C`` for the cost ``C`` it is asked for.

All numbers are dyadic rationals (``k / 2**s``) printed with their exact,
finite decimal expansion, so that a reader working in binary at any precision
(GMP ``mpf`` in the reference, the multi-limb format here) parses exactly the
same value.  Only the upper triangle (``i <= j``) of each symmetric matrix is
written, as SDPA does.

Problem families (sizes are parameters):

* ``maxcut``  -- MaxCut relaxation of an Erdos-Renyi graph: ``C = L/4``
  (graph Laplacian) as a maximisation, i.e. ``F0 = L/4``; ``F_i = e_i e_i^T``,
  ``c_i = 1``.  Unit weights or +-1 weights.
* ``gpp``     -- graph-partition type: ``F0 = -L``, ``F_i = e_i e_i^T`` with
  ``c_i = 1`` for ``i <= n`` plus ``F_{n+1} = 1 1^T`` with ``c = 0``.
* ``control`` -- control/LMI type with dense random constraint matrices on
  several blocks and a strictly feasible primal-dual pair built from
  ``X0 = Q diag(U[0.5,2]) Q^T`` and ``Z0`` likewise.
"""
from __future__ import annotations

import math
import os
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 200

_DYADIC_BITS = 24


def _dyadic(x: float, bits: int = _DYADIC_BITS) -> str:
    """Round ``x`` to ``k / 2**bits`` and return the exact decimal string."""
    k = int(round(x * (1 << bits)))
    if k == 0:
        return "0"
    d = Decimal(k) / Decimal(1 << bits)
    s = format(d, "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def _exact(num: int, den_pow2: int) -> str:
    """Exact decimal of ``num / 2**den_pow2``."""
    if num == 0:
        return "0"
    d = Decimal(num) / Decimal(1 << den_pow2)
    s = format(d, "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


class SDPText:
    """Accumulates a ``.dat-s`` problem: ``F0..Fm`` entries and ``c``."""

    def __init__(self, title: str, m: int, block_struct: list[int]):
        self.title = title
        self.m = m
        self.block_struct = list(block_struct)
        self.c: list[str] = ["0"] * m
        self.entries: list[tuple[int, int, int, int, str]] = []

    def add(self, k: int, block: int, i: int, j: int, value: str) -> None:
        """Add entry (i, j) (1-based, any order) of block ``block`` (1-based) of F_k."""
        if value in ("0", "-0"):
            return
        if i > j:
            i, j = j, i
        self.entries.append((k, block, i, j, value))

    def text(self) -> str:
        out = [f'"{self.title}"', f"{self.m} = mDIM", f"{len(self.block_struct)} = nBLOCK",
               " ".join(str(b) for b in self.block_struct) + " = bLOCKsTRUCT",
               " ".join(self.c)]
        for k, b, i, j, v in self.entries:
            out.append(f"{k} {b} {i} {j} {v}")
        return "\n".join(out) + "\n"

    def write(self, path: str) -> str:
        with open(path, "w") as f:
            f.write(self.text())
        return path


def _er_graph(n: int, p: float, rng: np.random.Generator, signed: bool):
    edges = []
    for i in range(n):
        r = rng.random(n - i - 1)
        w = rng.random(n - i - 1)
        for t, j in enumerate(range(i + 1, n)):
            if r[t] < p:
                wt = (1 if w[t] < 0.5 else -1) if signed else 1
                edges.append((i, j, wt))
    return edges


def maxcut(n: int = 100, p: float = 0.1, seed: int = 0, signed: bool = False) -> SDPText:
    """MaxCut relaxation, ``max (L/4).X s.t. diag(X) = 1``; m = n."""
    rng = np.random.default_rng(seed)
    edges = _er_graph(n, p, rng, signed)
    deg = np.zeros(n, dtype=np.int64)
    prob = SDPText(f"maxcut n={n} p={p} seed={seed} signed={int(signed)}", n, [n])
    lap_off = {}
    for i, j, w in edges:
        deg[i] += w
        deg[j] += w
        lap_off[(i, j)] = lap_off.get((i, j), 0) - w
    # F0 = L/4 (maximisation of (L/4).X == minimisation of -(L/4).X, C = -F0)
    for i in range(n):
        prob.add(0, 1, i + 1, i + 1, _exact(int(deg[i]), 2))
    for (i, j), v in lap_off.items():
        prob.add(0, 1, i + 1, j + 1, _exact(v, 2))
    for i in range(n):
        prob.c[i] = "1"
        prob.add(i + 1, 1, i + 1, i + 1, "1")
    return prob


def gpp(n: int = 500, p: float = 0.02, seed: int = 0) -> SDPText:
    """Graph-partition type: ``C = -L`` as the SDPA ``F0``, diag(X)=1, (11^T).X = 0."""
    rng = np.random.default_rng(seed)
    edges = _er_graph(n, p, rng, False)
    deg = np.zeros(n, dtype=np.int64)
    m = n + 1
    prob = SDPText(f"gpp n={n} p={p} seed={seed}", m, [n])
    for i, j, w in edges:
        deg[i] += w
        deg[j] += w
    # F0 = -L: diagonal -deg, off-diagonal +w for each edge
    for i in range(n):
        prob.add(0, 1, i + 1, i + 1, str(-int(deg[i])))
    for i, j, w in edges:
        prob.add(0, 1, i + 1, j + 1, str(int(w)))
    for i in range(n):
        prob.c[i] = "1"
        prob.add(i + 1, 1, i + 1, i + 1, "1")
    prob.c[n] = "0"
    for i in range(n):
        for j in range(i, n):
            prob.add(n + 1, 1, i + 1, j + 1, "1")
    return prob


def _haar(n: int, rng: np.random.Generator) -> list[list[float]]:
    """Haar-distributed orthogonal matrix (rows) by modified Gram-Schmidt of a
    Gaussian matrix, with every dot product exactly rounded (``math.fsum``) so
    the result is identical on every platform (no BLAS/LAPACK summation order)."""
    g = rng.standard_normal((n, n))
    cols = [[float(g[i, j]) for i in range(n)] for j in range(n)]
    q: list[list[float]] = []
    for v in cols:
        w = list(v)
        for u in q:
            d = math.fsum(a * b for a, b in zip(u, w))
            w = [a - d * b for a, b in zip(w, u)]
        nrm = math.sqrt(math.fsum(a * a for a in w))
        q.append([a / nrm for a in w])
    return q  # q[k] is the k-th orthonormal column


def _spd(n: int, rng: np.random.Generator) -> list[list[float]]:
    """``Q diag(U[0.5, 2]) Q^T`` with exactly rounded sums."""
    q = _haar(n, rng)
    lam = [float(x) for x in rng.uniform(0.5, 2.0, n)]
    return [[math.fsum(lam[k] * q[k][a] * q[k][b] for k in range(n)) for b in range(n)]
            for a in range(n)]


def control(m: int = 231, blocks: tuple[int, ...] = (40, 20), seed: int = 0) -> SDPText:
    """Control/LMI type: dense symmetric N(0,1) constraints on every block.

    ``X0 = Q diag(U[0.5,2]) Q^T`` gives ``b_i = tr(A_i X0)``; ``y0 ~ N(0,1)`` and
    ``Z0`` (built like ``X0``) give ``C = Z0 + sum_i y0_i A_i``, so
    ``(X0, y0, Z0)`` is a strictly feasible primal-dual triple of
    ``min C.X s.t. A_i.X = b_i``.  Written as SDPA data: ``F0 = -C``.
    All sums are exactly rounded, so the file is byte-identical everywhere.
    """
    return _control(m, blocks, seed)


def control_lp(m: int = 30, blocks: tuple[int, ...] = (12,), lp: int = 10, density: float = 0.3,
               seed: int = 0) -> SDPText:
    """`control` with an LP block of `lp` nonnegative variables appended (block size
    -lp in the file): every constraint gets N(0,1) coefficients on a random `density`
    share of them (at least one); ``x0, z0 ~ U[0.5, 2]`` extend the strictly feasible
    triple with the same ``y0``.  Sums exactly rounded: byte-identical everywhere."""
    return _control(m, blocks, seed, lp=lp, density=density)


def _control(m, blocks, seed, lp: int = 0, density: float = 0.3) -> SDPText:
    rng = np.random.default_rng(seed)
    if lp:
        prob = SDPText(f"control_lp m={m} blocks={list(blocks)} lp={lp} seed={seed}", m, list(blocks) + [-lp])
    else:
        prob = SDPText(f"control m={m} blocks={list(blocks)} seed={seed}", m, list(blocks))
    scale = float(1 << _DYADIC_BITS)
    A = []  # A[l][i] = list of upper-triangle values, row-major over (a <= b)
    for nb in blocks:
        Ab = []
        for _ in range(m):
            g = rng.standard_normal((nb, nb))
            Ab.append([[round((float(g[a, b]) + float(g[b, a])) / math.sqrt(2.0) * scale) / scale
                        for b in range(nb)] for a in range(nb)])
        A.append(Ab)
    X0 = [_spd(nb, rng) for nb in blocks]
    y0 = [float(x) for x in rng.standard_normal(m)]
    Z0 = [_spd(nb, rng) for nb in blocks]
    coef, x0, z0 = [], [], []
    if lp:  # drawn after everything `control` draws, so its blocks are unchanged
        for _ in range(m):
            mask = rng.random(lp) < density
            mask[int(rng.integers(0, lp))] = True
            vals = rng.standard_normal(lp)
            coef.append({k: round(float(vals[k]) * scale) / scale for k in range(lp) if mask[k]})
        x0 = [float(v) for v in rng.uniform(0.5, 2.0, lp)]
        z0 = [float(v) for v in rng.uniform(0.5, 2.0, lp)]
    for i in range(m):
        terms = []
        for l, nb in enumerate(blocks):
            Ai, Xl = A[l][i], X0[l]
            for a in range(nb):
                for b in range(nb):
                    s_ab = Ai[min(a, b)][max(a, b)]
                    terms.append(s_ab * Xl[a][b])
        if lp:
            terms += [a * x0[k] for k, a in coef[i].items()]
        prob.c[i] = _dyadic(math.fsum(terms))
    for l, nb in enumerate(blocks):
        for a in range(nb):
            for b in range(a, nb):
                c_ab = math.fsum([Z0[l][a][b]] + [y0[i] * A[l][i][a][b] for i in range(m)])
                prob.add(0, l + 1, a + 1, b + 1, _dyadic(-c_ab))
    for i in range(m):
        for l, nb in enumerate(blocks):
            Ai = A[l][i]
            for a in range(nb):
                for b in range(a, nb):
                    prob.add(i + 1, l + 1, a + 1, b + 1, _dyadic(Ai[a][b]))
    if lp:
        lpb = len(blocks) + 1
        for k in range(lp):  # C = z0 + sum_i y0_i a_i on the LP block (F0 = -C)
            c_k = math.fsum([z0[k]] + [y0[i] * coef[i][k] for i in range(m) if k in coef[i]])
            prob.add(0, lpb, k + 1, k + 1, _dyadic(-c_k))
        for i in range(m):
            for k, a in sorted(coef[i].items()):
                prob.add(i + 1, lpb, k + 1, k + 1, _dyadic(a))
    return prob


def param_text(precision: int = 256, max_iteration: int = 200, epsilon_star: str = "1.0E-30",
               lambda_star: str = "1.0E4", beta_star: str = "0.1", beta_bar: str = "0.3",
               gamma_star: str = "0.9", epsilon_dash: str = "1.0E-30", print_format: str = "%+50.40Fe") -> str:
    """A ``param.sdpa`` file in the reference's 15-line positional layout
    (Parameter::readFile, sdpa_parts.cpp:188-225); defaults are the reference's
    default parameter set (sdpa_parts.cpp:163-176) except ``precision``.
    ``print_format`` is the GMP format of xVec / xMat / yMat (lines 12-14; at most
    29 characters, the reference's buffer)."""
    return (f"{max_iteration}\tunsigned int maxIteration;\n"
            f"{epsilon_star}\tdouble 0.0 < epsilonStar;\n"
            f"{lambda_star}   double 0.0 < lambdaStar;\n"
            f"2.0   \tdouble 1.0 < omegaStar;\n"
            f"-1.0E5  double lowerBound;\n"
            f"1.0E5   double upperBound;\n"
            f"{beta_star}     double 0.0 <= betaStar <  1.0;\n"
            f"{beta_bar}     double 0.0 <= betaBar  <  1.0, betaStar <= betaBar;\n"
            f"{gamma_star}     double 0.0 < gammaStar  <  1.0;\n"
            f"{epsilon_dash}\tdouble 0.0 < epsilonDash;\n"
            f"{precision}     precision\n"
            f"{print_format}     char*  xPrint   (default %+8.3e,   NOPRINT skips printout)\n"
            f"{print_format}     char*  XPrint   (default %+8.3e,   NOPRINT skips printout)\n"
            f"{print_format}     char*  YPrint   (default %+8.3e,   NOPRINT skips printout)\n"
            "%+50.40Fe     char*  infPrint (default %+10.16e, NOPRINT skips printout)\n")


WORKLOADS = {
    # name: (constructor, kwargs, precision)
    "maxcut100": (maxcut, dict(n=100, p=0.1, seed=0), 256),
    "control231": (control, dict(m=231, blocks=(40, 20), seed=0), 256),
    "gpp500": (gpp, dict(n=500, p=0.02, seed=0), 256),
    "gpp500_p512": (gpp, dict(n=500, p=0.02, seed=0), 512),
    "maxcut124pm": (maxcut, dict(n=124, p=0.1, seed=0, signed=True), 256),
}


def write_workload(name: str, directory: str) -> tuple[str, str]:
    """Write ``<name>.dat-s`` and ``<name>.param`` into ``directory``."""
    ctor, kw, prec = WORKLOADS[name]
    os.makedirs(directory, exist_ok=True)
    dat = ctor(**kw).write(os.path.join(directory, f"{name}.dat-s"))
    par = os.path.join(directory, f"{name}.param")
    with open(par, "w") as f:
        f.write(param_text(precision=prec))
    return dat, par


def _spd_np(n: int, rng: np.random.Generator) -> np.ndarray:
    """Q diag(U[0.5, 2]) Q^T with Q Haar-orthogonal (numpy sums)."""
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    q = q * np.sign(np.diag(r))
    lam = rng.uniform(0.5, 2.0, n)
    return (q * lam) @ q.T


def control_dense(m: int, blocks, rng: np.random.Generator):
    """The control/LMI construction of `control` with numpy sums, returned as dense
    arrays for Problem.from_dense (c, F0 blocks, F blocks of shape (m, n, n)); entries
    are dyadic (k / 2^24).  Not byte-identical across machines (BLAS sums); used for
    the batched workload, whose instances are generated where they are solved."""
    scale = float(1 << _DYADIC_BITS)
    dy = lambda x: np.round(x * scale) / scale  # noqa: E731
    F = []
    for nb in blocks:
        g = rng.standard_normal((m, nb, nb))
        F.append(dy((g + g.transpose(0, 2, 1)) / math.sqrt(2.0)))
    X0 = [_spd_np(nb, rng) for nb in blocks]
    y0 = rng.standard_normal(m)
    Z0 = [_spd_np(nb, rng) for nb in blocks]
    c = dy(sum(np.einsum("iab,ab->i", F[l], X0[l]) for l in range(len(blocks))))
    F0 = [dy(-(Z0[l] + np.tensordot(y0, F[l], axes=1))) for l in range(len(blocks))]
    F0 = [(b + b.T) / 2 for b in F0]  # exactly symmetric (the halves are dyadic)
    return c, F0, F


def batch_instance_size(seed: int) -> tuple[int, list[int]]:
    """(m, block sizes) of batch_instance(seed), from the same first draws, without
    building the instance."""
    rng = np.random.default_rng(seed)
    m = int(rng.integers(20, 351))
    blocks = [int(x) for x in rng.integers(15, 91, size=2)]
    return m, blocks


def batch_instance(seed: int):
    """One instance of the batched workload: m ~ U[20, 350], two blocks of sizes
    ~ U[15, 90], control/LMI construction, all drawn from `seed`."""
    rng = np.random.default_rng(seed)
    m = int(rng.integers(20, 351))
    blocks = [int(x) for x in rng.integers(15, 91, size=2)]
    return control_dense(m, blocks, rng)
