"""GB300 multi-limb SDPA Newton-step library: Python mirror of the C ABI.

``libsdpg.so`` (built in-tree by ``build.py``) holds every kernel and the
solver; this module only loads it through ctypes and converts arguments.
There is no CPU fallback: if the library is missing, importing ``lib``
raises.  Number arrays use the library's own element layout (see
``include/sdpg.h``): a numpy ``uint32`` array of shape ``(count, limbs + 2)``
holding ``[e, s, m[0], ..., m[limbs-1]]`` per value, column-major for matrices.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libsdpg.so")

# A solve keeps four streams busy (batched solves many more); CUDA reads this when the
# context is created, so it only takes effect if nothing in the process has used CUDA yet.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_SQRT = 0, 1, 2, 3, 4


class SdpgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sdpg error {code}: {msg}")
        self.code = code


_lib = None


class Param(ctypes.Structure):
    """Interior-point parameters (the reference's Parameter, sdpa_parts.cpp:136-225)."""
    _fields_ = [("maxIteration", ctypes.c_int), ("epsilonStar", ctypes.c_double),
                ("lambdaStar", ctypes.c_double), ("omegaStar", ctypes.c_double),
                ("lowerBound", ctypes.c_double), ("upperBound", ctypes.c_double),
                ("betaStar", ctypes.c_double), ("betaBar", ctypes.c_double),
                ("gammaStar", ctypes.c_double), ("epsilonDash", ctypes.c_double),
                ("precision", ctypes.c_int)]

    @classmethod
    def default(cls, preset: int = 0) -> "Param":
        p = cls()
        check(lib().sdpg_param_default(ctypes.byref(p), preset))
        return p

    @classmethod
    def read(cls, path: str) -> "Param":
        p = cls.default()
        check(lib().sdpg_param_read(ctypes.byref(p), path.encode()))
        return p


def _setup(lib: ctypes.CDLL) -> ctypes.CDLL:
    c = ctypes
    vp, i, ll, ch = c.c_void_p, c.c_int, c.c_longlong, c.c_char
    sig = {
        "sdpg_last_error": (c.c_char_p, []),
        "sdpg_version": (i, []),
        "sdpg_limbs_for_precision": (i, [i]),
        "sdpg_ml_elem_bytes": (i, [i]),
        "sdpg_ml_parse": (i, [i, c.c_char_p, vp]),
        "sdpg_ml_format": (i, [i, vp, i, c.c_char_p, i]),
        "sdpg_ml_format_gmp": (i, [i, vp, c.c_char_p, c.c_char_p, i]),
        "sdpg_ml_from_double": (i, [i, vp, ll, vp]),
        "sdpg_ml_to_double": (i, [i, vp, ll, vp]),
        "sdpg_ml_from_mpf": (i, [i, vp, ll, vp]),
        "sdpg_ml_to_mpf": (i, [i, vp, ll, vp]),
        "sdpg_ml_host_op": (i, [i, i, ll, vp, vp, vp]),
        "sdpg_rgemm": (i, [i, ch, ch, i, i, i, vp, vp, i, vp, i, vp, vp, i]),
        "sdpg_rgemm_device": (i, [i, ch, ch, i, i, i, vp, vp, i, vp, i, vp, vp, i, vp]),
        "sdpg_rpotrf": (i, [i, i, vp, i, c.POINTER(i)]),
        "sdpg_inv_lower": (i, [i, i, vp, i, vp]),
        "sdpg_solve_systems": (i, [i, i, vp, i, vp]),
        "sdpg_tridiag_min": (i, [i, i, vp, vp, vp]),
        "sdpg_sym_min_eigen": (i, [i, i, vp, vp]),
        "sdpg_param_default": (i, [c.POINTER(Param), i]),
        "sdpg_param_read": (i, [c.POINTER(Param), c.c_char_p]),
        "sdpg_problem_new": (vp, [i, i, c.POINTER(i), c.POINTER(i)]),
        "sdpg_problem_read": (vp, [c.c_char_p, i, c.POINTER(i)]),
        "sdpg_problem_free": (None, [vp]),
        "sdpg_problem_set_c": (i, [vp, i, c.c_char_p]),
        "sdpg_problem_add_entry": (i, [vp, i, i, i, i, c.c_char_p]),
        "sdpg_problem_add_entry_mpf": (i, [vp, i, i, i, i, vp]),
        "sdpg_problem_set_c_double": (i, [vp, i, c.c_double]),
        "sdpg_problem_add_dense": (i, [vp, i, i, i, vp]),
        "sdpg_solve_batch": (i, [i, vp, c.POINTER(Param), i, i, vp, vp]),
        "sdpg_solver_create": (vp, [vp, c.POINTER(Param), i, vp, c.POINTER(i)]),
        "sdpg_solver_destroy": (None, [vp]),
        "sdpg_solver_limbs": (i, [vp]),
        "sdpg_solver_dims": (i, [vp, c.POINTER(i), c.POINTER(i), c.POINTER(i), i]),
        "sdpg_solver_initialize": (i, [vp]),
        "sdpg_solver_run": (i, [vp, c.c_char_p, i]),
        "sdpg_solver_iterate": (i, [vp]),
        "sdpg_newton": (i, [vp, i]),
        "sdpg_step_length": (i, [vp, i]),
        "sdpg_update": (i, [vp]),
        "sdpg_residuals": (i, [vp]),
        "sdpg_make_schur": (i, [vp, vp]),
        "sdpg_make_gvec": (i, [vp, i, vp]),
        "sdpg_min_eigen": (i, [vp, i, vp]),
        "sdpg_solution_info": (i, [vp, c.POINTER(c.c_double)]),
        "sdpg_solution_text": (i, [vp, i, i, c.c_char_p, i]),
        "sdpg_get_xvec": (i, [vp, i, vp]),
        "sdpg_get_block": (i, [vp, i, i, i, vp]),
        "sdpg_get_vector": (i, [vp, i, vp]),
        "sdpg_solver_timers": (i, [vp, c.POINTER(c.c_double)]),
        "sdpg_solver_history": (i, [vp, c.POINTER(c.c_double), i]),
        "sdpg_solver_gemm_macs": (c.c_longlong, [vp]),
        "sdpg_solver_reset_counters": (i, [vp]),
        "sdpg_solver_gemm_profile": (i, [vp, i, c.POINTER(c.c_double)]),
        "sdpg_solver_io_bytes": (i, [vp, c.POINTER(ll), c.POINTER(ll)]),
        "sdpg_launch_count": (c.c_ulonglong, []),
        "sdpg_set_gemm_method": (i, [i]),
        "sdpg_tensor_error": (i, [i, c.POINTER(i)]),
        "sdpg_set_tensor_wait_budget": (ll, [ll]),
        "sdpg_kernel_timing": (i, [i]),
        "sdpg_kernel_times": (i, [c.c_char_p, i]),
        "sdpg_probe_imad_wide": (i, [i, c.POINTER(c.c_double)]),
        "sdpg_probe_tensor_rate": (i, [i, i, c.POINTER(c.c_double)]),
        "sdpg_solve_file": (i, [c.c_char_p, c.c_char_p, c.c_char_p, i, c.POINTER(c.c_double)]),
        "sdpg_policy_create": (i, [i, c.POINTER(vp)]),
        "sdpg_policy_destroy": (None, [vp]),
        "sdpg_policy_set": (i, [vp, vp, vp]),
        "sdpg_policy_get": (i, [vp, vp, vp]),
        "sdpg_policy_forward": (i, [vp, vp, i, vp]),
        "sdpg_policy_gradient": (i, [vp, vp, vp, vp, i, vp, vp]),
        "sdpg_policy_train": (i, [vp, vp, vp, vp, i, i, i, c.c_float, c.c_ulonglong, vp]),
        "sdpg_solver_set_policy": (i, [vp, vp, i]),
        "sdpg_solver_read_initial_point": (i, [vp, c.c_char_p, i]),
        "sdpg_solve_file_ex": (i, [c.c_char_p, i, c.POINTER(Param), c.c_char_p, c.c_char_p, i, c.c_char_p, i, i,
                                   c.POINTER(c.c_double)]),
        "sdpg_solver_policy_stats": (i, [vp, c.POINTER(c.c_double)]),
        "sdpg_solver_features": (i, [vp, vp, i]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    return lib


def lib() -> ctypes.CDLL:
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built: run build.py (no CPU fallback exists)")
        _lib = _setup(ctypes.CDLL(LIB_PATH))
    return _lib


def check(rc: int) -> int:
    if rc < 0:
        raise SdpgError(rc, lib().sdpg_last_error().decode())
    return rc


def limbs_for_precision(bits: int) -> int:
    return check(lib().sdpg_limbs_for_precision(bits))


def ml_empty(count: int, limbs: int) -> np.ndarray:
    return np.zeros((count, limbs + 2), dtype=np.uint32)


def ml_parse(texts, limbs: int) -> np.ndarray:
    """Decimal strings -> ml array (exact up to truncation at the format's precision)."""
    texts = list(texts)
    out = ml_empty(len(texts), limbs)
    for k, t in enumerate(texts):
        check(lib().sdpg_ml_parse(limbs, t.encode(), out[k].ctypes.data))
    return out


def ml_from_double(x, limbs: int) -> np.ndarray:
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
    out = ml_empty(x.size, limbs)
    check(lib().sdpg_ml_from_double(limbs, x.ctypes.data, x.size, out.ctypes.data))
    return out


def ml_to_double(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    limbs = a.shape[1] - 2
    out = np.zeros(a.shape[0], dtype=np.float64)
    check(lib().sdpg_ml_to_double(limbs, a.ctypes.data, a.shape[0], out.ctypes.data))
    return out


def ml_format(a: np.ndarray, digits: int = 17) -> list[str]:
    a = np.ascontiguousarray(a)
    limbs = a.shape[1] - 2
    buf = ctypes.create_string_buffer(digits + 32)
    res = []
    for k in range(a.shape[0]):
        check(lib().sdpg_ml_format(limbs, a[k].ctypes.data, digits, buf, len(buf)))
        res.append(buf.value.decode())
    return res


def ml_format_gmp(a: np.ndarray, fmt: str) -> list[str]:
    """Each value through a GMP printf format such as "%+50.40Fe" (the result file's)."""
    limbs = a.shape[1] - 2
    a = np.ascontiguousarray(a)
    buf = ctypes.create_string_buffer(4096)
    out = []
    for row in a:
        check(lib().sdpg_ml_format_gmp(limbs, row.ctypes.data, fmt.encode(), buf, len(buf)))
        out.append(buf.value.decode())
    return out


def ml_host_op(op: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a)
    b = a if b is None else np.ascontiguousarray(b)
    limbs = a.shape[1] - 2
    out = np.empty_like(a)
    check(lib().sdpg_ml_host_op(limbs, op, a.shape[0], a.ctypes.data, b.ctypes.data, out.ctypes.data))
    return out


def rgemm(transa: str, transb: str, m: int, n: int, k: int, alpha: np.ndarray, A: np.ndarray, lda: int,
          B: np.ndarray, ldb: int, beta: np.ndarray, C: np.ndarray, ldc: int) -> np.ndarray:
    """``C = alpha op(A) op(B) + beta C`` on the GPU (Rgemm signature); returns the new C."""
    limbs = A.shape[1] - 2
    A = np.ascontiguousarray(A)
    B = np.ascontiguousarray(B)
    C = np.array(C, copy=True, order="C")
    alpha = np.ascontiguousarray(alpha).reshape(-1)
    beta = np.ascontiguousarray(beta).reshape(-1)
    check(lib().sdpg_rgemm(limbs, transa.encode(), transb.encode(), m, n, k, alpha.ctypes.data,
                           A.ctypes.data, lda, B.ctypes.data, ldb, beta.ctypes.data, C.ctypes.data, ldc))
    return C


def rpotrf(A: np.ndarray, n: int, lda: int) -> tuple[np.ndarray, int]:
    """Lower Cholesky in place on a copy (Rpotrf "Lower"); returns (factor, info)."""
    limbs = A.shape[1] - 2
    A = np.array(A, copy=True, order="C")
    info = ctypes.c_int(0)
    check(lib().sdpg_rpotrf(limbs, n, A.ctypes.data, lda, ctypes.byref(info)))
    return A, info.value


def inv_lower(L: np.ndarray, n: int, ldl: int) -> np.ndarray:
    """L^{-1} (n x n, ld n) of a lower-triangular L."""
    limbs = L.shape[1] - 2
    L = np.ascontiguousarray(L)
    out = ml_empty(n * n, limbs)
    check(lib().sdpg_inv_lower(limbs, n, L.ctypes.data, ldl, out.ctypes.data))
    return out


def solve_systems(L: np.ndarray, n: int, ldl: int, x: np.ndarray) -> np.ndarray:
    """(L L^T)^{-1} x."""
    limbs = L.shape[1] - 2
    L = np.ascontiguousarray(L)
    x = np.array(x, copy=True, order="C")
    check(lib().sdpg_solve_systems(limbs, n, L.ctypes.data, ldl, x.ctypes.data))
    return x


def tridiag_min(d: np.ndarray, e: np.ndarray) -> np.ndarray:
    """Smallest eigenvalue of tridiag(e, d, e) and the last component of its eigenvector."""
    limbs = d.shape[1] - 2
    d = np.ascontiguousarray(d)
    e = np.ascontiguousarray(e if len(e) else ml_empty(1, limbs))
    out = ml_empty(2, limbs)
    check(lib().sdpg_tridiag_min(limbs, d.shape[0], d.ctypes.data, e.ctypes.data, out.ctypes.data))
    return out


def sym_min_eigen(A: np.ndarray, n: int) -> np.ndarray:
    """Smallest eigenvalue of a dense symmetric n x n (n <= 64)."""
    limbs = A.shape[1] - 2
    A = np.ascontiguousarray(A)
    out = ml_empty(2, limbs)
    check(lib().sdpg_sym_min_eigen(limbs, n, A.ctypes.data, out.ctypes.data))
    return out[:1]


PHASES = ["noINFO", "pFEAS", "dFEAS", "pdFEAS", "pdINF", "pFEAS_dINF", "pINF_dFEAS", "pdOPT", "pUNBD",
          "dUNBD"]
INFO_KEYS = ["phase", "iteration", "objValPrimal", "objValDual", "mu", "relative gap", "p.feas.error",
             "d.feas.error", "alphaP", "alphaD", "beta", "digits"]


class Problem:
    """SDPA problem data (F_0..F_m, c), 1-based indices as in .dat-s files."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def read(cls, path: str, dense: bool = False) -> "Problem":
        err = ctypes.c_int(0)
        h = lib().sdpg_problem_read(path.encode(), 1 if dense else 0, ctypes.byref(err))
        if not h:
            check(err.value)
        return cls(h)

    @classmethod
    def new(cls, m: int, block_struct) -> "Problem":
        bs = (ctypes.c_int * len(block_struct))(*block_struct)
        err = ctypes.c_int(0)
        h = lib().sdpg_problem_new(m, len(block_struct), bs, ctypes.byref(err))
        if not h:
            check(err.value)
        return cls(h)

    def set_c(self, k: int, value) -> None:
        check(lib().sdpg_problem_set_c(self.h, k, str(value).encode()))

    def add_entry(self, k: int, block: int, i: int, j: int, value) -> None:
        check(lib().sdpg_problem_add_entry(self.h, k, block, i, j, str(value).encode()))

    def set_c_double(self, k: int, value: float) -> None:
        check(lib().sdpg_problem_set_c_double(self.h, k, float(value)))

    def add_dense(self, k: int, block: int, A: np.ndarray) -> None:
        """Upper triangle of the dense symmetric block `block` of F_k (doubles, exact)."""
        A = np.asfortranarray(A, dtype=np.float64)
        check(lib().sdpg_problem_add_dense(self.h, k, block, A.shape[0], A.ctypes.data))

    @classmethod
    def from_dense(cls, c, F0, F) -> "Problem":
        """min c.x  s.t.  sum_i F_i x_i - F0 >= 0, with dense symmetric blocks:
        c (m,), F0 list of (n_l, n_l), F list over blocks of (m, n_l, n_l)."""
        m = len(c)
        blocks = [int(b.shape[0]) for b in F0]
        prob = cls.new(m, blocks)
        for k in range(m):
            prob.set_c_double(k + 1, float(c[k]))
        for l, b in enumerate(F0):
            prob.add_dense(0, l + 1, b)
            for k in range(m):
                prob.add_dense(k + 1, l + 1, F[l][k])
        return prob

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.sdpg_problem_free(self.h)
            self.h = None


class Solver:
    """GPU-resident interior-point solver (one problem, one stream)."""

    def __init__(self, problem: Problem, param: Param | None = None, device: int = 0, stream: int = 0):
        param = param or Param.default()
        err = ctypes.c_int(0)
        self.h = lib().sdpg_solver_create(problem.h, ctypes.byref(param), device, stream or None,
                                          ctypes.byref(err))
        if not self.h:
            check(err.value)
        self.limbs = check(lib().sdpg_solver_limbs(self.h))
        m, nb = ctypes.c_int(), ctypes.c_int()
        sizes = (ctypes.c_int * 4096)()
        check(lib().sdpg_solver_dims(self.h, ctypes.byref(m), ctypes.byref(nb), sizes, 4096))
        self.m = m.value
        self.block_sizes = [sizes[i] for i in range(nb.value)]

    def close(self) -> None:
        if getattr(self, "h", None) and _lib is not None:
            _lib.sdpg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def initialize(self) -> None:
        check(lib().sdpg_solver_initialize(self.h))

    def run(self, out_path: str | None = None, verbose: bool = False) -> int:
        return check(lib().sdpg_solver_run(self.h, out_path.encode() if out_path else None, 1 if verbose else 0))

    def iterate(self) -> bool:
        """One predictor-corrector iteration; False once the solve has stopped."""
        return check(lib().sdpg_solver_iterate(self.h)) == 1

    def newton(self, direction: int) -> bool:
        rc = lib().sdpg_newton(self.h, direction)
        if rc == -3:
            return False
        check(rc)
        return True

    def step_length(self, direction: int) -> None:
        check(lib().sdpg_step_length(self.h, direction))

    def update(self) -> bool:
        rc = lib().sdpg_update(self.h)
        if rc == -3:
            return False
        check(rc)
        return True

    def residuals(self) -> None:
        check(lib().sdpg_residuals(self.h))

    def info(self) -> dict:
        out = (ctypes.c_double * 12)()
        check(lib().sdpg_solution_info(self.h, out))
        d = dict(zip(INFO_KEYS, list(out)))
        d["phase"] = PHASES[int(d["phase"])]
        d["iteration"] = int(d["iteration"])
        return d

    def text(self, which: int, digits: int = 40) -> str:
        buf = ctypes.create_string_buffer(digits + 32)
        check(lib().sdpg_solution_text(self.h, which, digits, buf, len(buf)))
        return buf.value.decode()

    def xvec(self, ml: bool = False) -> np.ndarray:
        if ml:
            out = ml_empty(self.m, self.limbs)
            check(lib().sdpg_get_xvec(self.h, 1, out.ctypes.data))
            return out
        out = np.zeros(self.m)
        check(lib().sdpg_get_xvec(self.h, 0, out.ctypes.data))
        return out

    def block(self, which: int, l: int, ml: bool = False) -> np.ndarray:
        n = self.block_sizes[l]
        if ml:
            out = ml_empty(n * n, self.limbs)
            check(lib().sdpg_get_block(self.h, which, l, 1, out.ctypes.data))
            return out
        out = np.zeros(n * n)
        check(lib().sdpg_get_block(self.h, which, l, 0, out.ctypes.data))
        return out.reshape(n, n, order="F")

    def vector(self, which: int) -> np.ndarray:
        out = ml_empty(self.m, self.limbs)
        check(lib().sdpg_get_vector(self.h, which, out.ctypes.data))
        return out

    def schur(self) -> np.ndarray:
        out = ml_empty(self.m * self.m, self.limbs)
        check(lib().sdpg_make_schur(self.h, out.ctypes.data))
        return out

    def gvec(self, direction: int = 0) -> np.ndarray:
        out = ml_empty(self.m, self.limbs)
        check(lib().sdpg_make_gvec(self.h, direction, out.ctypes.data))
        return out

    def min_eigen(self, side: int) -> np.ndarray:
        out = ml_empty(1, self.limbs)
        check(lib().sdpg_min_eigen(self.h, side, out.ctypes.data))
        return out

    def timers(self) -> dict:
        out = (ctypes.c_double * 8)()
        check(lib().sdpg_solver_timers(self.h, out))
        return dict(zip(["schur", "cholesky", "rmat_gvec", "dxdz", "steplen", "update", "residual", "total"],
                        list(out)))

    def history(self) -> np.ndarray:
        out = (ctypes.c_double * (9 * 4096))()
        n = check(lib().sdpg_solver_history(self.h, out, 4096))
        return np.array(list(out)[: 9 * n]).reshape(n, 9)

    def gemm_macs(self) -> int:
        return int(lib().sdpg_solver_gemm_macs(self.h))

    def reset_counters(self) -> None:
        check(lib().sdpg_solver_reset_counters(self.h))

    def gemm_profile(self, enable: int = -1) -> dict:
        out = (ctypes.c_double * 3)()
        check(lib().sdpg_solver_gemm_profile(self.h, enable, out))
        return {"kernel_ms": out[0], "launches": int(out[1]), "macs": int(out[2])}

    def io_bytes(self) -> tuple[int, int]:
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().sdpg_solver_io_bytes(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def read_initial_point(self, path: str, sparse: bool = True) -> None:
        """Start the next initialize() from an -is (sparse) / -id (dense) initial-point file."""
        check(lib().sdpg_solver_read_initial_point(self.h, path.encode(), 1 if sparse else 0))

    def set_policy(self, policy: "Policy | None", beta: bool = True, lam: bool = True) -> None:
        """Attach a learned proposal (the policy must outlive the solver's use of it)."""
        self._policy = policy  # keep it alive
        flags = (1 if beta else 0) | (2 if lam else 0)
        check(lib().sdpg_solver_set_policy(self.h, policy.h if policy else None, flags if policy else 0))

    def policy_stats(self) -> dict:
        out = (ctypes.c_double * 4)()
        check(lib().sdpg_solver_policy_stats(self.h, out))
        return {"proposals": int(out[0]), "fallbacks": int(out[1]), "lambda_star": out[2],
                "lambda_proposed": out[3]}

    def features(self) -> np.ndarray:
        """Policy inputs: row 0 at the initial point, row k + 1 at iteration k."""
        n = check(lib().sdpg_solver_features(self.h, None, 0))
        out = np.zeros((max(n, 1), POLICY_INPUTS), dtype=np.float32)
        check(lib().sdpg_solver_features(self.h, out.ctypes.data, n))
        return out[:n]


POLICY_INPUTS = 6
POLICY_OUTPUTS = 2
POLICY_PARAMS = 8898
POLICY_SCALE = 16


class Policy:
    """The learned lambdaStar / beta proposal: a 6-64-64-64-2 tanh network in FP32 whose
    forward, backward and Adam steps run as the library's CUDA kernels."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().sdpg_policy_create(device, ctypes.byref(h)))
        self.h = h.value
        self.device = device

    def close(self) -> None:
        if getattr(self, "h", None) and _lib is not None:
            _lib.sdpg_policy_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def get(self) -> tuple[np.ndarray, np.ndarray]:
        w = np.zeros(POLICY_PARAMS, dtype=np.float32)
        sc = np.zeros(POLICY_SCALE, dtype=np.float32)
        check(lib().sdpg_policy_get(self.h, w.ctypes.data, sc.ctypes.data))
        return w, sc

    def set(self, params: np.ndarray | None = None, scale: np.ndarray | None = None) -> None:
        w = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        sc = None if scale is None else np.ascontiguousarray(scale, dtype=np.float32)
        if w is not None and w.size != POLICY_PARAMS:
            raise ValueError(f"expected {POLICY_PARAMS} parameters")
        if sc is not None and sc.size != POLICY_SCALE:
            raise ValueError(f"expected {POLICY_SCALE} scaling values")
        check(lib().sdpg_policy_set(self.h, None if w is None else w.ctypes.data,
                                    None if sc is None else sc.ctypes.data))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, POLICY_INPUTS)
        y = np.zeros((x.shape[0], POLICY_OUTPUTS), dtype=np.float32)
        check(lib().sdpg_policy_forward(self.h, x.ctypes.data, x.shape[0], y.ctypes.data))
        return y

    def gradient(self, x: np.ndarray, t: np.ndarray, mask: np.ndarray) -> tuple[np.ndarray, float]:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, POLICY_INPUTS)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, POLICY_OUTPUTS)
        mask = np.ascontiguousarray(mask, dtype=np.float32).reshape(-1, POLICY_OUTPUTS)
        g = np.zeros(POLICY_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        check(lib().sdpg_policy_gradient(self.h, x.ctypes.data, t.ctypes.data, mask.ctypes.data, x.shape[0],
                                         g.ctypes.data, ctypes.byref(loss)))
        return g, loss.value

    def train(self, x: np.ndarray, t: np.ndarray, mask: np.ndarray, epochs: int, batch: int = 256,
              lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, POLICY_INPUTS)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, POLICY_OUTPUTS)
        mask = np.ascontiguousarray(mask, dtype=np.float32).reshape(-1, POLICY_OUTPUTS)
        losses = np.zeros(max(epochs, 1), dtype=np.float32)
        check(lib().sdpg_policy_train(self.h, x.ctypes.data, t.ctypes.data, mask.ctypes.data, x.shape[0], epochs,
                                      batch, lr, seed, losses.ctypes.data))
        return losses[:epochs]

    def save(self, path: str) -> None:
        w, sc = self.get()
        np.savez(path, params=w, scale=sc)

    @classmethod
    def load(cls, path: str, device: int = 0) -> "Policy":
        d = np.load(path)
        p = cls(device)
        p.set(d["params"], d["scale"])
        return p


def set_gemm_method(method: int) -> int:
    """0: tensor-core residue path for 256-bit GEMMs where it applies; 1: digit GEMM only;
    2: residue path for every 256-bit GEMM with K <= 16384.  Returns the previous method."""
    return check(lib().sdpg_set_gemm_method(method))


def tensor_error(device: int = 0) -> int:
    flag = ctypes.c_int(0)
    check(lib().sdpg_tensor_error(device, ctypes.byref(flag)))
    return flag.value


def set_tensor_wait_budget(cycles: int) -> int:
    """Test hook: budget (clock cycles) of the tensor-core kernel's primary waits and the
    Cholesky panel's row waits; 0 restores the default.  Returns the previous setting."""
    return int(lib().sdpg_set_tensor_wait_budget(cycles))


def kernel_timing(enable: bool) -> bool:
    """Per-kernel CUDA-event timing on (graphs become plain launches) or off; returns the old state."""
    return bool(lib().sdpg_kernel_timing(1 if enable else 0))


def kernel_times() -> dict:
    """{kernel name: (launches, milliseconds, algorithmic work)} recorded since the last call."""
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().sdpg_kernel_times(buf, len(buf)))
    out = {}
    for ln in buf.value.decode().splitlines():
        name, cnt, ms, work = ln.split()
        out[name] = (int(cnt), float(ms), float(work))
    return out


def solve_batch(problems, param: Param | None = None, device: int = 0, concurrency: int = 16):
    """Solve many problems with up to `concurrency` solvers in flight on the GPU.
    Returns (iterations, info): iterations[i] < 0 is the error code of a failed solve;
    info[i] holds the 12 summary values of Solver.info() in INFO_KEYS order."""
    n = len(problems)
    handles = (ctypes.c_void_p * max(n, 1))(*[p.h for p in problems])
    info = np.zeros((max(n, 1), 12), dtype=np.float64)
    its = np.zeros(max(n, 1), dtype=np.int32)
    prm = param if param is not None else Param.default()
    check(lib().sdpg_solve_batch(n, handles, ctypes.byref(prm), device, concurrency, info.ctypes.data,
                                 its.ctypes.data))
    return its[:n], info[:n]


def launch_count() -> int:
    return int(lib().sdpg_launch_count())


def probe_imad_wide(device: int = 0) -> float:
    """Measured IMAD.WIDE (signed 32x32->64 multiply-add) operations per second."""
    out = ctypes.c_double()
    check(lib().sdpg_probe_imad_wide(device, ctypes.byref(out)))
    return out.value


TENSOR_PROBE_KINDS = {0: "tcgen05.mma kind::f16 (fp16 x fp16 -> fp32), M128 N256",
                      1: "mma.sync m16n8k32 s8 x s8 -> s32",
                      2: "mma.sync m16n8k16 f16 x f16 -> f32"}


def probe_tensor_rate(kind: int, device: int = 0) -> float:
    """Measured multiply-add operations (2 per MAC) per second of one tensor instruction
    (TENSOR_PROBE_KINDS) from fixed operands, no memory traffic."""
    out = ctypes.c_double()
    check(lib().sdpg_probe_tensor_rate(device, kind, ctypes.byref(out)))
    return out.value


def solve_file(data_path: str, param_path: str | None = None, out_path: str | None = None,
               device: int = 0) -> dict:
    """``sdpa_gmp -ds data -o out -p param`` on the GPU; returns the final info."""
    out = (ctypes.c_double * 12)()
    check(lib().sdpg_solve_file(data_path.encode(), param_path.encode() if param_path else None,
                                out_path.encode() if out_path else None, device, out))
    d = dict(zip(INFO_KEYS, list(out)))
    d["phase"] = PHASES[int(d["phase"])]
    d["iteration"] = int(d["iteration"])
    return d
