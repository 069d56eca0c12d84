"""Which tcgen05 product kinds the sm_103a target accepts (CPU only: the compiler, no GPU).

The residue GEMM multiplies fp16 residues (tcgen05.mma kind::f16) rather than 8-bit
integer slices: the compiler rejects tcgen05.mma kind::i8 for sm_103a, while it accepts
kind::f16 there (and kind::i8 for sm_100a).  The measured rates of the instructions that
do exist are in test_tensor_rate_gpu.py.
"""
import os
import shutil
import subprocess

import pytest

KERNEL = r"""
#include <stdint.h>
__global__ void k(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}
"""


def compile_kind(kind: str, arch: str, tmp) -> subprocess.CompletedProcess:
    src = os.path.join(tmp, f"k_{kind}_{arch}.cu")
    with open(src, "w") as f:
        f.write(KERNEL.replace("KIND", kind))
    return subprocess.run(["nvcc", f"-gencode=arch=compute_{arch},code=sm_{arch}", "-c", src, "-o",
                           src[:-3] + ".o"], capture_output=True, text=True)


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_int8_tensor_kind_absent_on_sm103a(tmp_path):
    f16 = compile_kind("f16", "103a", str(tmp_path))
    assert f16.returncode == 0, f16.stderr
    i8 = compile_kind("i8", "103a", str(tmp_path))
    assert i8.returncode != 0
    assert "not supported on .target 'sm_103a'" in i8.stderr, i8.stderr
    # the same instruction is accepted for the B200 target: the rejection is the target's
    i8_100 = compile_kind("i8", "100a", str(tmp_path))
    assert i8_100.returncode == 0, i8_100.stderr
