"""Per-thread resources of the CUDA kernels, from ptxas's own report (no GPU needed).

A kernel that copies an argument struct indexed at run time into local memory gets a
stack frame of the struct's size in every thread: the one-block coarse-level kernel once
had a 2672-byte frame that way, 1024 threads of one SM writing and reading 2.7 MB of
local memory per V-cycle (2.6x its time). Register spills of a few tens of bytes are
tuning choices (blocks per SM asked of the allocator); frames of kilobytes are bugs.
Every translation unit is compiled for sm_103a with -Xptxas -v, and every kernel's stack
frame must stay under 256 bytes; the one-block coarse kernel and the FP32 right-hand side
are also held to their current register budgets.
"""
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "nyles_gb300", "csrc")
MAX_FRAME = 256


def _ptxas_report(src, tmp):
    from nyles_gb300 import build
    cmd = [build.nvcc(), "-c", os.path.join(CSRC, src), "-o", os.path.join(tmp, src + ".o")] + build.ARCH + \
        build.FLAGS + ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stderr


def _kernels(report):
    """{mangled kernel name: (stack frame bytes, registers)} from a ptxas -v report"""
    out, cur, frame = {}, None, 0
    for line in report.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            cur, frame = m.group(1), 0
            continue
        m = re.search(r"(\d+) bytes stack frame", line)
        if m and cur:
            frame = int(m.group(1))
        m = re.search(r"Used (\d+) registers", line)
        if m and cur:
            out[cur] = (frame, int(m.group(1)))
            cur = None
    return out


@pytest.fixture(scope="module")
def kernels():
    try:
        from nyles_gb300 import build
        build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    tmp = tempfile.mkdtemp(prefix="nyles_ptxas_")
    try:
        srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
        with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
            reports = list(ex.map(lambda s: _ptxas_report(s, tmp), srcs))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    out = {}
    for rep in reports:
        out.update(_kernels(rep))
    return out


def test_no_kernel_has_a_large_stack_frame(kernels):
    assert len(kernels) > 50
    big = {k: v for k, v in kernels.items() if v[0] >= MAX_FRAME}
    assert not big, big


def test_hot_kernel_register_budgets(kernels):
    def find(fragment):
        hits = [v for k, v in kernels.items() if fragment in k]
        assert hits, fragment
        return hits
    # the one-block coarse levels (1024 threads: at most 64 registers) without a frame
    for frame, regs in find("k_mg_bottomIf"):
        assert frame == 0 and regs <= 64, (frame, regs)
    # the FP32 right-hand side at 5 blocks of 256 threads per SM (48 registers)
    for frame, regs in find("k_rhs_les"):
        assert regs <= 48, regs
