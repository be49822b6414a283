"""Every kernel of the library begins with dependent_launch_enter() (CPU, source check).

The solver joins consecutive kernels of its captured iteration by programmatic
graph edges (csrc/solver.cu, make_dependent_edges); a kernel so reached may be
scheduled while its predecessor still runs and must wait for it before its
first memory access.  That wait is dependent_launch_enter(), the first
statement of each kernel body.
"""
import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parent.parent / "mlpcg_gb300" / "csrc"


def _kernels(src):
    """(name, first statement of the body) of every __global__ definition in src."""
    for m in re.finditer(r"__global__", src):
        j = m.end()
        while True:
            mm = re.compile(r"[A-Za-z_]\w*\s*\(").search(src, j)
            name = mm.group(0).rstrip("( \n")
            k, depth = mm.end(), 1
            while depth:
                depth += {"(": 1, ")": -1}.get(src[k], 0)
                k += 1
            if name != "__launch_bounds__":
                break
            j = k
        rest = src[k:].lstrip()
        if not rest.startswith("{"):
            continue  # a declaration
        yield name, rest[1:].lstrip().split(";", 1)[0] + ";"


def test_every_kernel_waits_for_its_predecessor_first():
    found = 0
    for f in sorted(CSRC.glob("*.cu")):
        for name, first in _kernels(f.read_text()):
            found += 1
            assert first == "dependent_launch_enter();", (f.name, name, first)
    assert found > 50
