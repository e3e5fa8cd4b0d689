"""The C ABI library: loads, exports every entry point declared in
include/rskel.h, validates arguments and orders calls without touching a GPU,
and refuses to compute (no CPU fallback) when no GPU is present."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "rskel.h")).read()
    names = set(re.findall(r"^\s*(?:rs_status|void|const char\s*\*)\s*(rs_\w+)\s*\(", text,
                           re.MULTILINE))
    return sorted(names)


def test_library_exports_every_declared_symbol(solver_lib):
    lib = solver_lib.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(solver_lib.EXPORTS) == set(names)


def test_config_defaults_are_the_reference_defaults(solver_lib):
    c = solver_lib.default_config()
    assert c.id_tol == 1e-6 and c.max_leaf_dofs == 32 and c.num_proxy_points == 128
    assert c.radius_ratio == 1.5 and c.min_dofs_to_compress == 16
    assert c.is_strong_admissibility == 0 and c.solution_dimension == 1
    # fields beyond the reference's configuration
    assert c.precision == solver_lib.RS_FP64 and c.refine_verify == 1 and c.refine_solver == 0
    assert c.use_graphs == 1 and c.root_inverse == 1
    assert c.fmm_order32 == 0 and c.tensor_cores == 1 and c.id_row_groups == -1


def test_geometry_checks_leave_the_handle_unchanged(solver_lib):
    """A rejected geometry (non-finite weight) leaves the handle's previous
    geometry and tree in place: the check runs before anything changes."""
    from rskel import geometry as g

    s = solver_lib.Solver(g.unit_circle(20000), solver_lib.RS_LAPLACE, 1e-6)
    s.build_tree()
    before = s.tree_dump()
    bad = g.unit_circle(20000)
    bad.weights[123] = np.inf
    with pytest.raises(solver_lib.RsError) as e:
        s.set_geometry(bad)
    assert e.value.code == 6
    after = s.tree_dump()
    for k in ("level_sizes", "node_parent", "nbr", "orig"):
        assert np.array_equal(before[k], after[k]), k


def test_argument_validation(solver_lib):
    from rskel import geometry as g

    lib = solver_lib.lib()
    h = ctypes.c_void_p()
    bad = solver_lib.default_config(pde=2, solution_dimension=1)  # Stokes needs sd = 2
    assert lib.rs_create(ctypes.byref(bad), ctypes.byref(h)) == 1
    bad = solver_lib.default_config(id_tol=0.0)
    assert lib.rs_create(ctypes.byref(bad), ctypes.byref(h)) == 1
    bad = solver_lib.default_config(is_strong_admissibility=1)
    assert lib.rs_create(ctypes.byref(bad), ctypes.byref(h)) == 1
    # the FP32 correction products' multipole order: 0 (chosen per correction) or 2..16
    for o32, ok in ((0, True), (1, False), (2, True), (16, True), (17, False), (-1, False)):
        cfg = solver_lib.default_config(fmm_order32=o32)
        rc = lib.rs_create(ctypes.byref(cfg), ctypes.byref(h))
        assert (rc == 0) == ok, (o32, rc)
        if rc == 0:
            lib.rs_destroy(h)
    geo = g.unit_circle(64)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-6)
    with pytest.raises(solver_lib.RsError) as e:
        s.solve(np.ones(64))
    assert e.value.code == 2  # solve before factor
    with pytest.raises(solver_lib.RsError):
        s.kernel_block([0, 64], [1])  # index out of range
    # non-finite geometry is rejected before any compute
    geo.points[3] = np.nan
    with pytest.raises(solver_lib.RsError) as e:
        solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-6)
    assert e.value.code == 6


def _has_gpu():
    try:
        lib = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob

            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            lib = ctypes.CDLL(cands[0]) if cands else None
        except OSError:
            lib = None
    if lib is None:
        return False
    n = ctypes.c_int(0)
    return lib.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


def test_no_cpu_fallback_without_gpu(solver_lib):
    if _has_gpu():
        pytest.skip("a GPU is present")
    from rskel import geometry as g

    s = solver_lib.Solver(g.unit_circle(256), solver_lib.RS_LAPLACE, 1e-6)
    s.build_tree()  # host-side, works without a GPU
    with pytest.raises(solver_lib.RsError) as e:
        s.factor()
    assert e.value.code == 4  # RS_ERR_NO_DEVICE


def test_ctypes_structs_match_the_header(solver_lib, tmp_path):
    """The Python binding's rs_config and rs_stats mirrors have the header's
    layout: every field at the C compiler's offset, and the same size."""
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "rskel.h"', "int main(void) {"]
    for st, cname in ((solver_lib.RsConfig, "rs_config"), (solver_lib.RsStats, "rs_stats")):
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in st._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    res = subprocess.run(["gcc", "-I", inc, str(src), "-o", exe], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for st, cname in ((solver_lib.RsConfig, "rs_config"), (solver_lib.RsStats, "rs_stats")):
        assert got[(cname, "size")] == ctypes.sizeof(st), cname
        for f, _ in st._fields_:
            assert got[(cname, f)] == getattr(st, f).offset, (cname, f)
