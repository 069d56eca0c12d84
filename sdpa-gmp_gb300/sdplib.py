"""Sweep over problem / result pairs laid out like the reference's SDPLIB/data directory:
``<name>.dat-s`` (or ``.dat-s.xz``) beside the result file the reference wrote for it,
``<name>.result`` (or ``.result.xz``; SDPLIB/go.sh:95-102 produced the shipped ones).

For every pair found in a directory the parameters are taken from the result file's
parameter block (the lines after "Parameters are", sdpa_io.cpp's printout of
Parameter::display), the problem is solved on the GPU with them, and the final phase,
iteration count and objectives are compared with the recorded ones; the recorded main
loop time sits beside this solver's.  Nothing is bundled: the runner reads whatever
directory it is given.

    python -m sdpa-gmp_gb300.sdplib DIR [--only NAME ...] [--max-m M] [--json OUT]
"""
from __future__ import annotations

import argparse
import importlib
import json
import lzma
import os
import re
import sys
import tempfile
import time

_NUM = r"[-+]?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?"
PARAM_KEYS = ("maxIteration", "epsilonStar", "lambdaStar", "omegaStar", "lowerBound", "upperBound", "betaStar",
              "betaBar", "gammaStar", "epsilonDash", "precision")


def read_text(path: str) -> str:
    """A text file, decompressed when it ends in .xz."""
    if path.endswith(".xz"):
        with lzma.open(path, "rt") as f:
            return f.read()
    with open(path) as f:
        return f.read()


def parse_result(text: str) -> dict:
    """Phase, iteration count, objectives, parameters and times of a reference result file."""
    out: dict = {}
    m = re.search(r"phase\.value\s*=\s*(\S+)", text)
    if not m:
        raise ValueError("not a result file: no phase.value line")
    out["phase"] = m.group(1)
    for key, pat in (("iteration", r"Iteration\s*=\s*(\d+)"), ("objValPrimal", rf"objValPrimal\s*=\s*({_NUM})"),
                     ("objValDual", rf"objValDual\s*=\s*({_NUM})"), ("relative_gap", rf"relative gap\s*=\s*({_NUM})"),
                     ("total_time", rf"total time\s*=\s*({_NUM})"),
                     ("main_loop_time", rf"Main Loop\s*=\s*({_NUM})")):
        m = re.search(pat, text)
        if m:
            out[key] = int(m.group(1)) if key == "iteration" else float(m.group(1))
    params = {}
    block = text.split("Parameters are", 1)
    if len(block) == 2:
        for key in PARAM_KEYS:
            m = re.search(rf"\b{key}\s*=\s*({_NUM})", block[1])
            if m:
                params[key] = int(float(m.group(1))) if key in ("maxIteration", "precision") else float(m.group(1))
    out["params"] = params
    return out


def pairs(directory: str) -> list[tuple[str, str, str]]:
    """(name, data path, result path) for every problem with a result beside it, sorted."""
    files = set(os.listdir(directory))
    found = []
    for f in sorted(files):
        for ext in (".dat-s.xz", ".dat-s"):
            if f.endswith(ext):
                name = f[: -len(ext)]
                res = next((r for r in (name + ".result.xz", name + ".result") if r in files), None)
                if res:
                    found.append((name, os.path.join(directory, f), os.path.join(directory, res)))
    # a name with both a compressed and a plain data file counts once
    seen, out = set(), []
    for t in found:
        if t[0] not in seen:
            seen.add(t[0])
            out.append(t)
    return out


def data_size(text: str) -> tuple[int, list[int]]:
    """m and the block structure from the head of a .dat-s text (comment lines skipped)."""
    lines = [ln for ln in text.splitlines() if ln.strip() and ln.lstrip()[0] not in "\"*"]
    m = int(re.findall(r"[-+]?\d+", lines[0])[0])
    nblock = int(re.findall(r"[-+]?\d+", lines[1])[0])
    blocks = [int(v) for v in re.findall(r"[-+]?\d+", lines[2])[:nblock]]
    return m, blocks


def param_from(sdpg, params: dict):
    """The solver's parameter set for a result file's parameter block (defaults elsewhere)."""
    p = sdpg.Param.default()
    for key, v in params.items():
        setattr(p, key, v)
    return p


def run_case(sdpg, name: str, data_path: str, result_path: str, device: int = 0) -> dict:
    ref = parse_result(read_text(result_path))
    text = read_text(data_path)
    with tempfile.TemporaryDirectory() as tmp:
        dat = os.path.join(tmp, name + ".dat-s")
        with open(dat, "w") as f:
            f.write(text)
        t0 = time.perf_counter()
        solver = sdpg.Solver(sdpg.Problem.read(dat), param_from(sdpg, ref["params"]), device=device)
        solver.run()
        secs = time.perf_counter() - t0
    info = solver.info()
    row = {"name": name, "reference": {k: ref.get(k) for k in ("phase", "iteration", "objValPrimal", "objValDual",
                                                              "main_loop_time")},
           "ours": {"phase": info["phase"], "iteration": info["iteration"], "objValPrimal": info["objValPrimal"],
                    "objValDual": info["objValDual"], "seconds": secs},
           "precision": ref["params"].get("precision")}
    rel = lambda a, b: abs(a - b) / max(1.0, abs(b))  # noqa: E731
    row["same_phase"] = info["phase"] == ref["phase"]
    row["iteration_difference"] = info["iteration"] - ref["iteration"]
    row["objective_rel_difference"] = max(rel(info["objValPrimal"], ref["objValPrimal"]),
                                          rel(info["objValDual"], ref["objValDual"]))
    return row


def sweep(directory: str, only=None, max_m: int | None = None, device: int = 0, log=None) -> list[dict]:
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    rows = []
    for name, dat, res in pairs(directory):
        if only and name not in only:
            continue
        if max_m is not None and data_size(read_text(dat))[0] > max_m:
            continue
        try:
            row = run_case(sdpg, name, dat, res, device)
        except Exception as exc:  # the sweep goes on; the row records the failure
            row = {"name": name, "error": f"{type(exc).__name__}: {exc}"}
        rows.append(row)
        if log:
            log(row)
    return rows


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("directory")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--max-m", type=int, default=None, help="skip problems with more constraints")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--json", default=None, help="write all rows to this file")
    a = ap.parse_args(argv)

    def log(r):
        if "error" in r:
            print(f"{r['name']:>14s}  ERROR {r['error']}")
            return
        o, f = r["ours"], r["reference"]
        print(f"{r['name']:>14s}  {o['phase']:>7s}/{f['phase']:<7s} it {o['iteration']:3d}/{f['iteration']:<3d} "
              f"obj rel diff {r['objective_rel_difference']:.1e}  {o['seconds']:8.2f} s (reference main loop "
              f"{f['main_loop_time']} s)", flush=True)

    rows = sweep(a.directory, a.only, a.max_m, a.device, log)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rows, f, indent=1)
    bad = [r for r in rows if "error" in r or not r["same_phase"]]
    print(f"{len(rows)} problems, {len(bad)} with an error or another final phase")
    return 0 if not bad else 1


if __name__ == "__main__":
    sys.exit(main())
