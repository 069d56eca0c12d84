"""Generate the golden fixtures in tests/golden/ by running the reference
solver itself (oracle/_ref/sdpa_gmp, built from the reference sources by
oracle/build_ref.sh) on seeded synthetic problems and on the reference's own
known-answer input (example1.dat-s).

This script runs only where the reference sources exist (it builds the
binary from them); the GPU-side tests read the JSON it writes and regenerate
the same ``.dat-s`` text from the package's generators, checking its sha256.

Each fixture records what the reference prints: the per-iteration table
(mu, thetaP, thetaD, objP, objD, alphaP, alphaD, beta), the final block
(phase, iteration count, mu, gaps, objectives, feasibility errors) and the
final primal vector ``xVec`` to 40 significant digits (``%+50.40Fe``).

Usage: python tests/golden/make_golden.py [--only NAME ...] [--ref DIR] [--precise]
(--ref defaults to $SDPG_REFERENCE_DIR, else /root/reference)
"""
from __future__ import annotations

import argparse
import hashlib
import importlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
problems = importlib.import_module("sdpa-gmp_gb300.problems")

# name -> (generator, kwargs, precision, max_iteration)
CASES = {
    "maxcut20": ("maxcut", dict(n=20, p=0.3, seed=1), 256),
    "maxcut40": ("maxcut", dict(n=40, p=0.2, seed=2), 256),
    "maxcut40_p512": ("maxcut", dict(n=40, p=0.2, seed=2), 512),
    "maxcut40pm": ("maxcut", dict(n=40, p=0.15, seed=3, signed=True), 256),
    "control20": ("control", dict(m=20, blocks=(10, 6), seed=2), 256),
    "control30": ("control", dict(m=30, blocks=(24, 12), seed=1), 256),
    "gpp40": ("gpp", dict(n=40, p=0.1, seed=1), 256),
    "gpp60": ("gpp", dict(n=60, p=0.08, seed=4), 256),
    "maxcut100": ("maxcut", dict(n=100, p=0.1, seed=0), 256),
    "maxcut124pm": ("maxcut", dict(n=124, p=0.1, seed=0, signed=True), 256),
    "control231": ("control", dict(m=231, blocks=(40, 20), seed=0), 256),
    # LP blocks (a fourth element would hold param_text overrides)
    "controllp20": ("control_lp", dict(m=20, blocks=(10,), lp=12, seed=5), 256),
    "controllp40": ("control_lp", dict(m=40, blocks=(24, 8), lp=30, density=0.2, seed=6), 256),
}

# High-precision cases: the reference prints xVec / xMat / yMat with `print_format`
# (param.sdpa lines 12-14), so its final iterate is known to far below 2^-p.  The
# fixture keeps xVec, the objectives recomputed exactly from the printed solution
# (c.x and F0.Y), and for large blocks only the first column and diagonal of xMat /
# yMat.  max_iteration < 200 stops the reference after that many iterations, which
# gives fixed-iteration comparisons of the same run.
P80 = "%+.80Fe"
P160 = "%+.160Fe"
P200 = "%+.200Fe"
PRECISE = {
    "gpp500_hp": ("gpp", dict(n=500, p=0.02, seed=0), 256, dict(print_format=P80)),
    "gpp500_it5": ("gpp", dict(n=500, p=0.02, seed=0), 256, dict(print_format=P80, max_iteration=5)),
    "gpp500_it10": ("gpp", dict(n=500, p=0.02, seed=0), 256, dict(print_format=P80, max_iteration=10)),
    "gpp500_it20": ("gpp", dict(n=500, p=0.02, seed=0), 256, dict(print_format=P80, max_iteration=20)),
    "gpp500_p512_it10": ("gpp", dict(n=500, p=0.02, seed=0), 512, dict(print_format=P160, max_iteration=10)),
    # the same ten iterations at 1024 bits: a yardstick for both the 256- and 512-bit runs
    "gpp500_p1024_it10": ("gpp", dict(n=500, p=0.02, seed=0), 1024, dict(print_format=P200, max_iteration=10)),
    "control231_hp": ("control", dict(m=231, blocks=(40, 20), seed=0), 256, dict(print_format=P80)),
    "maxcut124pm_hp": ("maxcut", dict(n=124, p=0.1, seed=0, signed=True), 256, dict(print_format=P80)),
    "maxcut100_hp": ("maxcut", dict(n=100, p=0.1, seed=0), 256, dict(print_format=P80)),
}
FULL_MATRIX_LIMIT = 4000  # larger solutions keep only a digest

ITER_RE = re.compile(r"^\s*(\d+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s*$")
FINAL_KEYS = ["mu", "relative gap", "gap", "digits", "objValPrimal", "objValDual",
              "p.feas.error", "d.feas.error", "relative eps"]


def parse_result(text: str) -> dict:
    lines = text.splitlines()
    out: dict = {"iterations_table": []}
    i = 0
    while i < len(lines) and not lines[i].lstrip().startswith("mu "):
        i += 1
    i += 1
    while i < len(lines):
        mt = ITER_RE.match(lines[i])
        if not mt:
            break
        out["iterations_table"].append(list(mt.groups()))
        i += 1
    for ln in lines:
        if ln.startswith("phase.value"):
            out["phase"] = ln.split("=")[1].strip()
        elif ln.strip().startswith("Iteration ="):
            out["iteration"] = int(ln.split("=")[1])
        else:
            for k in FINAL_KEYS:
                if ln.strip().startswith(k + " ") or ln.strip().startswith(k + "="):
                    lhs = ln.split("=")[0].strip()
                    if lhs == k:
                        out[k] = ln.split("=")[1].strip()
    xv = re.search(r"xVec = \n\{(.*?)\}\n", text, re.S)
    if xv:
        out["xVec"] = [s.strip() for s in xv.group(1).split(",")]
    for key, nxt in (("xMat", "yMat = "), ("yMat", "    main loop time")):
        mt = re.search(key + r" = \n(.*?)\n" + re.escape(nxt), text, re.S)
        if mt:
            out[key] = NUM_RE.findall(mt.group(1))
    out["layout"] = result_layout(text)
    return out


NUM_RE = re.compile(r"[+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|nan|inf)")


def result_layout(text: str) -> list[str]:
    """The result file's lines with every number replaced by '#' and the start time and
    file names masked: what must agree between two solvers' result files."""
    out = []
    for ln in text.splitlines():
        if ln.startswith("SDPA-GMP start at"):
            ln = "SDPA-GMP start at <time>"
        for tag in ("data      is ", "parameter is ", "initial   is ", "out       is "):
            if ln.startswith(tag):
                ln = tag + "<path>"
        out.append(NUM_RE.sub("#", ln))
    return out


def precise_fields(r: dict, prob, digits: int = 90) -> None:
    """Replace r's xMat / yMat by a digest when large and add the objectives computed
    exactly (decimal, 200 digits) from the printed solution: objValPrimal = c.xVec and
    objValDual = F0.yMat (SDPA's printed primal / dual, sdpa_io.cpp:1095-1109, 1166-1173),
    and the relative gap |P - D| / max(1, (|P| + |D|) / 2) (sdpa_io.cpp:1001-1003)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 2 * digits + 40
    x = [Decimal(v) for v in r["xVec"]]
    objp = sum(Decimal(c) * xi for c, xi in zip(prob.c, x))
    sizes = [abs(b) for b in prob.block_struct]
    offs, o = [], 0
    for b, nb in zip(prob.block_struct, sizes):
        offs.append(o)
        o += nb * nb if b > 0 else nb
    ymat = r["yMat"]
    assert len(ymat) == o, (len(ymat), o)

    def y(block, i, j):  # 1-based entry of block `block` of yMat
        b = prob.block_struct[block - 1]
        if b < 0:
            return Decimal(ymat[offs[block - 1] + i - 1]) if i == j else Decimal(0)
        return Decimal(ymat[offs[block - 1] + (i - 1) * sizes[block - 1] + (j - 1)])

    objd = Decimal(0)
    for k, blk, i, j, v in prob.entries:
        if k == 0:
            objd += Decimal(v) * y(blk, i, j) * (1 if i == j else 2)
    gap = abs(objp - objd) / max(Decimal(1), (abs(objp) + abs(objd)) / 2)
    r["objValPrimal_hp"] = format(objp, f".{digits}e")
    r["objValDual_hp"] = format(objd, f".{digits}e")
    r["relgap_hp"] = format(gap, f".{digits}e")
    if len(ymat) > FULL_MATRIX_LIMIT:
        dig = {}
        for key in ("xMat", "yMat"):
            vals = r.pop(key)
            d = {"diag": [], "col0": []}
            for blk, (b, nb) in enumerate(zip(prob.block_struct, sizes)):
                if b < 0:
                    continue
                base = offs[blk]
                d["diag"].append([vals[base + i * nb + i] for i in range(nb)])
                d["col0"].append([vals[base + i * nb] for i in range(nb)])
            dig[key] = d
        r["digest"] = dig
    r["layout"] = [ln for ln in r["layout"] if not ln.startswith("{")][:400]


def run_case(binary: str, dat_text: str, param_text: str, workdir: str, name: str, extra=()) -> dict:
    dat = os.path.join(workdir, name + ".dat-s")
    par = os.path.join(workdir, name + ".param")
    res = os.path.join(workdir, name + ".result")
    with open(dat, "w") as f:
        f.write(dat_text)
    with open(par, "w") as f:
        f.write(param_text)
    env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count() or 1))
    subprocess.run([binary, "-ds", dat, "-o", res, "-p", par, *extra], check=True, env=env,
                   stdout=subprocess.DEVNULL)
    with open(res) as f:
        return parse_result(f.read())


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--ref", default=os.environ.get("SDPG_REFERENCE_DIR", "/root/reference"))
    ap.add_argument("--precise", action="store_true", help="also run the high-precision cases")
    args = ap.parse_args()
    binary = os.path.join(ROOT, "oracle", "_ref", "sdpa_gmp")
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), args.ref], check=True,
                   stdout=subprocess.DEVNULL)
    work = tempfile.mkdtemp(prefix="sdpg_golden_")
    try:
        if not args.only or "example1" in args.only:
            shutil.copy(os.path.join(args.ref, "example1.dat-s"), os.path.join(HERE, "example1.dat-s"))
            with open(os.path.join(HERE, "example1.dat-s")) as f:
                dat_text = f.read()
            with open(os.path.join(args.ref, "param.sdpa")) as f:
                param_text = f.read()
            with open(os.path.join(HERE, "example1.param"), "w") as f:
                f.write(param_text)
            r = run_case(binary, dat_text, param_text, work, "example1")
            r.update(name="example1", source="reference example1.dat-s + param.sdpa",
                     precision=200, sha256=hashlib.sha256(dat_text.encode()).hexdigest())
            with open(os.path.join(HERE, "example1.json"), "w") as f:
                json.dump(r, f, indent=1)
            print("example1", r["phase"], r["iteration"], r["objValPrimal"])
            # the reference's own initial points for example1: sparse (-is) and dense (-id)
            for tag, fname, opt in (("is", "example1.ini-s", "-is"), ("id", "example1.ini", "-id")):
                shutil.copy(os.path.join(args.ref, fname), os.path.join(HERE, fname))
                r = run_case(binary, dat_text, param_text, work, "example1_" + tag,
                             extra=(opt, os.path.join(HERE, fname)))
                r.update(name="example1_" + tag, source=f"reference example1.dat-s + param.sdpa + {fname} ({opt})",
                         precision=200, sha256=hashlib.sha256(dat_text.encode()).hexdigest(),
                         init={"file": fname, "sparse": opt == "-is"})
                with open(os.path.join(HERE, "example1_" + tag + ".json"), "w") as f:
                    json.dump(r, f, indent=1)
                print("example1_" + tag, r["phase"], r["iteration"], r["objValPrimal"])
            # the same problem in the dense data format (-dd example1.dat)
            shutil.copy(os.path.join(args.ref, "example1.dat"), os.path.join(HERE, "example1.dat"))
            res = os.path.join(work, "example1_dd.result")
            subprocess.run([binary, "-dd", os.path.join(HERE, "example1.dat"), "-o", res, "-p",
                            os.path.join(HERE, "example1.param")], check=True, stdout=subprocess.DEVNULL)
            with open(res) as f:
                r = parse_result(f.read())
            r.update(name="example1_dd", source="reference example1.dat (-dd) + param.sdpa", precision=200)
            with open(os.path.join(HERE, "example1_dd.json"), "w") as f:
                json.dump(r, f, indent=1)
            print("example1_dd", r["phase"], r["iteration"], r["objValPrimal"])
        for name, case in CASES.items():
            if args.only and name not in args.only:
                continue
            gen, kw, prec = case[:3]
            pkw = case[3] if len(case) > 3 else {}
            dat_text = getattr(problems, gen)(**kw).text()
            param_text = problems.param_text(precision=prec, **pkw)
            r = run_case(binary, dat_text, param_text, work, name)
            r.update(name=name, generator=gen, kwargs={k: (list(v) if isinstance(v, tuple) else v)
                                                         for k, v in kw.items()},
                     precision=prec, sha256=hashlib.sha256(dat_text.encode()).hexdigest())
            if pkw:
                r["param"] = pkw
            with open(os.path.join(HERE, name + ".json"), "w") as f:
                json.dump(r, f, indent=1)
            print(name, r.get("phase"), r.get("iteration"), r.get("objValPrimal"))
        for name, (gen, kw, prec, pkw) in PRECISE.items():
            if not args.precise or (args.only and name not in args.only):
                continue
            prob = getattr(problems, gen)(**kw)
            dat_text = prob.text()
            param_text = problems.param_text(precision=prec, **pkw)
            t0 = time.time()
            r = run_case(binary, dat_text, param_text, work, name)
            # digits of the stored objectives: ten beyond the print format's
            precise_fields(r, prob, digits=int(pkw["print_format"].split(".")[1].rstrip("Fe")) + 10)
            r.update(name=name, generator=gen, kwargs={k: (list(v) if isinstance(v, tuple) else v)
                                                         for k, v in kw.items()},
                     precision=prec, sha256=hashlib.sha256(dat_text.encode()).hexdigest(), param=pkw,
                     reference_seconds=round(time.time() - t0, 1))
            with open(os.path.join(HERE, name + ".json"), "w") as f:
                json.dump(r, f, indent=0)
            print(name, r.get("phase"), r.get("iteration"), r["objValPrimal_hp"][:30], r["reference_seconds"], "s",
                  flush=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
