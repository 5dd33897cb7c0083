"""The Cython declarations of the C ABI (include/wbgpu.pxd), compiled.

tests/shim/node_partition.pyx is a compiled caller written against the .pxd,
as a proximity tree's builder would partition all the open nodes of a depth
through wb_nearest_pivot (tree/_cptree.pyx:869-894).  It is cythonized and
compiled against libwbgpu.so here; the CPU tests check that it binds and that
the library's validation and messages reach it, the GPU test that its
partition equals the Python binding's (wildboar_gb300.distance.batch).
"""

import os
import subprocess
import sys
import sysconfig

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    pytest.importorskip("Cython")
    from wildboar_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libwbgpu.so is not built")
    out = tmp_path_factory.mktemp("shim")
    c_file = out / "node_partition.c"
    subprocess.run([sys.executable, "-m", "cython", "-3", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "shim", "node_partition.pyx"), "-o",
                    str(c_file)], check=True, capture_output=True)
    so = out / ("node_partition" + sysconfig.get_config_var("EXT_SUFFIX"))
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["gcc", "-shared", "-fPIC", "-O2", f"-I{sysconfig.get_paths()['include']}",
           f"-I{os.path.join(ROOT, 'include')}", str(c_file), f"-L{libdir}", "-lwbgpu",
           f"-Wl,-rpath,{libdir}", "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    sys.path.insert(0, str(out))
    try:
        import node_partition
    finally:
        sys.path.remove(str(out))
    return node_partition


def _node_data():
    rng = np.random.default_rng(3)
    x = np.ascontiguousarray(np.cumsum(rng.standard_normal((30, 1, 40)), axis=-1))
    # two nodes: samples and pivots as rows of x (CSR), node 1 with dtw r=0.2
    sample_ptr = np.array([0, 10, 22], dtype=np.int64)
    samples = np.arange(8, 30, dtype=np.int64)
    pivot_ptr = np.array([0, 3, 8], dtype=np.int64)
    pivots = np.array([0, 1, 2, 3, 4, 5, 6, 7], dtype=np.int64)
    group_slot = np.array([0, 1], dtype=np.int32)
    slot_metric = np.array([0, 1], dtype=np.int32)  # euclidean, dtw
    slot_r = np.array([1.0, 0.2])
    return x, sample_ptr, samples, pivot_ptr, pivots, group_slot, slot_metric, slot_r


def test_shim_binds_the_library(shim):
    assert shim.version() == 1


def test_shim_receives_the_library_validation(shim):
    # checks that run before any device call: the status and the library's
    # message come back through the compiled caller
    x, sp, s, pp, p, gs, sm, sr = _node_data()
    st, msg, _, _ = shim.partition_nodes(x, sp, s, pp, p, gs, sm, sr, dim=3)
    assert st == 1 and msg == "dim out of range"


@pytest.mark.gpu
def test_shim_partition_matches_python_binding(shim):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from wildboar_gb300.distance.batch import nearest_pivot

    x, sp, s, pp, p, gs, sm, sr = _node_data()
    st, msg, branch, dist = shim.partition_nodes(x, sp, s, pp, p, gs, sm, sr)
    assert st == 0, msg
    groups = [(s[sp[g]:sp[g + 1]], p[pp[g]:pp[g + 1]], int(gs[g])) for g in range(2)]
    wb, wd = nearest_pivot(x, groups, [("euclidean", {}), ("dtw", {"r": 0.2})])
    np.testing.assert_array_equal(branch, wb)
    np.testing.assert_array_equal(dist, wd)


def test_pxd_declares_every_entry_of_the_header():
    # every prototype of include/wbgpu.h appears in include/wbgpu.pxd with the
    # same return type, name and parameter list (whitespace aside, "(void)"
    # written "()" as Cython does), so compiled callers can use the whole ABI
    import re

    def norm(text):
        return " ".join(text.split()).replace("( ", "(").replace(" )", ")")

    h = open(os.path.join(ROOT, "include", "wbgpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    protos = re.findall(r"^((?:int|int64_t|int32_t|const char \*|void)\s*\**\s*wb_\w+\s*"
                        r"\([^;]*\));", h, flags=re.M)
    assert len(protos) >= 38
    pxd = norm(open(os.path.join(ROOT, "include", "wbgpu.pxd")).read())
    missing = [p for p in protos if norm(p).replace("(void)", "()") not in pxd]
    assert not missing, missing
