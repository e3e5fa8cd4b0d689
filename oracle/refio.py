"""Problem/result files exchanged with oracle/ref_dump.cpp (the driver around
the reference solver built from its own sources into oracle/_ref/).

Test infrastructure only: used to pin the oracle restatement and to generate
the golden fixtures under tests/golden/.  See oracle/ref_dump.cpp for the
binary layout.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def write_problem(path, geo, pde, sd, rhs, tol, leaf, npp, threads=1, repeats=1,
                  dense_check=False):
    rhs = np.asarray(rhs, dtype=np.float64)
    if rhs.ndim == 1:
        rhs = rhs[:, None]
    n = geo.n
    assert rhs.shape[0] == n * sd
    with open(path, "wb") as f:
        f.write(b"RSPROB01")
        f.write(struct.pack("<10i", pde, sd, n, geo.num_holes, rhs.shape[1], leaf, npp,
                            threads, repeats, 1 if dense_check else 0))
        f.write(struct.pack("<d", tol))
        for arr in (geo.points, geo.normals, geo.weights, geo.curvatures,
                    geo.hole_centers, geo.hole_radii):
            f.write(np.ascontiguousarray(arr, dtype="<f8").tobytes())
        f.write(np.asfortranarray(rhs, dtype="<f8").tobytes(order="F"))


def read_result(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"RSRES001", "bad result file"
    pos = 8
    while pos < len(data):
        (ln,) = struct.unpack_from("<i", data, pos)
        pos += 4
        name = data[pos:pos + ln].decode()
        pos += ln
        dtype, cnt = struct.unpack_from("<iq", data, pos)
        pos += 12
        dt = np.int32 if dtype == 1 else np.float64
        nbytes = cnt * np.dtype(dt).itemsize
        out[name] = np.frombuffer(data[pos:pos + nbytes], dtype=dt).copy()
        pos += nbytes
    return out


def ref_binary(leaf, npp):
    path = os.path.join(REF_DIR, f"ref_dump_{leaf}_{npp}")
    return path if os.path.exists(path) else None


def run_reference(geo, pde, sd, rhs, tol, leaf=64, npp=64, threads=1, repeats=1,
                  dense_check=False, timeout=3600, strong=False):
    """Run the reference build on one problem; returns the result dict."""
    exe = ref_binary(leaf, npp)
    if exe is None:
        raise FileNotFoundError(f"reference build for leaf {leaf} / proxy {npp} missing "
                                f"(make -C oracle ref)")
    with tempfile.TemporaryDirectory() as td:
        pin = os.path.join(td, "p.rsp")
        pout = os.path.join(td, "r.rsr")
        write_problem(pin, geo, pde, sd, rhs, tol, leaf, npp, threads, repeats, dense_check)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
        cmd = [exe, pin, pout] + (["--strong"] if strong else [])
        subprocess.run(cmd, check=True, timeout=timeout, env=env)
        return read_result(pout)


def run_reference_id(mats, tols, leaf=64, npp=64):
    """Run the reference's ie_Mat::id (dgeqp3 + dtrtrs) on each matrix."""
    exe = ref_binary(leaf, npp)
    if exe is None:
        raise FileNotFoundError("reference build missing (make -C oracle ref)")
    with tempfile.TemporaryDirectory() as td:
        pin = os.path.join(td, "ids.bin")
        pout = os.path.join(td, "ids.rsr")
        with open(pin, "wb") as f:
            f.write(struct.pack("<i", len(mats)))
            for a, tol in zip(mats, tols):
                a = np.asfortranarray(a, dtype="<f8")
                f.write(struct.pack("<iid", a.shape[0], a.shape[1], tol))
                f.write(a.tobytes(order="F"))
        subprocess.run([exe, "--id", pin, pout], check=True, timeout=600)
        return read_result(pout)


def run_reference_perturb(geos, sd, leaf=32, npp=128, timeout=600):
    """The reference's QuadTree::initialize_tree on geos[0], then
    QuadTree::perturb with geos[1], geos[2], ... in turn; returns the final
    tree (the result-file fields of a solve run, without the solution)."""
    exe = ref_binary(leaf, npp)
    if exe is None:
        raise FileNotFoundError("reference build missing (make -C oracle ref)")
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for i, geo in enumerate(geos):
            pth = os.path.join(td, f"p{i}.rsp")
            write_problem(pth, geo, 0 if sd == 1 else 2, sd, np.zeros(geo.n * sd), 1e-8, leaf,
                          npp)
            paths.append(pth)
        pout = os.path.join(td, "r.rsr")
        subprocess.run([exe, "--perturb", *paths, pout], check=True, timeout=timeout)
        return read_result(pout)


def csr(res, name, i):
    off = res[name + "_off"]
    return res[name][off[i]:off[i + 1]]
