"""The C ABI without a GPU: the library loads, exports every function that
include/*.h declares, and its host tree builder reproduces the reference's
layout (fixtures made by the reference itself)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from golden_util import inputs_of

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**(tk_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("tk_tree_create", "tk_tree_query", "tk_tree_destroy", "tk_tree_get_perm", "tk_tree_get_points",
                 "tk_knn_backward", "tk_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from torch_kdtree_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert not [n for n in declared_functions() if n not in _lib.SIGNATURES]


C_PROGRAM = r"""
#include <stdio.h>
#include "tk_knn.h"
int main(void) {
    float pts[8 * 3];
    int32_t perm[8];
    float dists[2], q[3] = {0.f, 0.f, 0.f};
    int32_t idx[2];
    tk_tree* tree = NULL;
    tk_tree_info info;
    for (int i = 0; i < 8 * 3; ++i) pts[i] = (float)((i * 7) % 11);
    if (tk_tree_create(pts, 8, 3, TK_F32, 2, -1, 1, &tree) != TK_OK) return 1;  /* host-only tree */
    if (tk_tree_get_info(tree, &info) != TK_OK || info.n_points != 8 || info.dims != 3) return 2;
    if (tk_tree_get_perm(tree, perm) != TK_OK) return 3;
    /* queries need a device image: refused, with a message, never computed on the CPU */
    if (tk_tree_query_host(tree, q, 1, 2, dists, idx, NULL, TK_HOST_AUTO, NULL) != TK_EINVAL) return 4;
    if (tk_last_error()[0] == 0) return 5;
    tk_tree_destroy(tree);
    printf("ok %d\n", tk_version());
    return 0;
}
"""


def test_header_is_c99_and_links_from_c(tmp_path):
    """The boundary is plain C: the header compiles as strict C99 and a C
    program links against libtkknn.so and runs (host-only calls, no GPU)."""
    import shutil
    import subprocess
    from torch_kdtree_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use_tk.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "use_tk"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe), "-L", libdir, "-ltkknn", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.startswith("ok ")


def host_tree(points, levels):
    from torch_kdtree_gb300._lib import LIB
    h = ctypes.c_void_p()
    dt = 0 if points.dtype == np.float32 else 1
    st = LIB.tk_tree_create(points.ctypes.data, points.shape[0], points.shape[1], dt, levels, -1, 0,
                            ctypes.byref(h))
    return st, h


def layout_of(h, n, d, levels, dtype):
    from torch_kdtree_gb300._lib import LIB, check
    perm = np.empty(n, np.int32)
    pts = np.empty((n, d), dtype)
    med = np.empty((1 << levels) - 1, dtype)
    off = np.empty((1 << levels) + 1, np.int32)
    check(LIB.tk_tree_get_perm(h, perm.ctypes.data))
    check(LIB.tk_tree_get_points(h, pts.ctypes.data))
    check(LIB.tk_tree_get_splits(h, med.ctypes.data, off.ctypes.data))
    return pts, perm, med, off


@pytest.mark.parametrize("name", [
    "grid_f32_d1_n1000_q200_k10", "grid_f32_d2_n10000_q300_k20", "grid_f32_d3_n10000_q300_k20",
    "grid_f64_d1_n10000_q300_k20", "grid_f64_d3_n1000_q200_k10", "grid_f32_d3_n30_q20_k5",
    "grid_f64_d2_n5_q5_k1", "levels_f32_d3_n1000_L9", "levels_f32_d3_n1000_L1",
    # 4-8 dimensions (the reference's README recipe)
    "wide_f32_d4_n1000_q200_k10", "wide_f32_d5_n10000_q300_k20", "wide_f32_d8_n10000_q300_k16",
    "wide_f64_d6_n1000_q200_k10", "wide_f64_d8_n5000_q200_k33", "wide_f32_d7_n30_q20_k5"])
def test_host_build_matches_reference_layout(name, golden):
    from torch_kdtree_gb300._lib import LIB, check
    case = golden[name]
    ref, _ = inputs_of(case)
    n, d = ref.shape
    L = int(case["levels"])
    st, h = host_tree(ref, L)
    check(st)
    try:
        pts, perm, med, off = layout_of(h, n, d, L, ref.dtype)
    finally:
        LIB.tk_tree_destroy(h)
    np.testing.assert_array_equal(pts, case["structured"])
    np.testing.assert_array_equal(perm, case["perm"])
    np.testing.assert_array_equal(med, case["medians"])
    depth = np.floor(np.log2(np.arange(len(med)) + 1)).astype(int)
    np.testing.assert_array_equal(depth % d, case["axes"])
    np.testing.assert_array_equal(off[:-1], case["leaf_off"])
    np.testing.assert_array_equal(np.diff(off), case["leaf_cnt"])


def test_host_build_matches_oracle_on_large_cloud(oracle):
    """Selection-based build == the oracle's full-sort build at 200k points."""
    from torch_kdtree_gb300._lib import LIB, check
    rng = np.random.default_rng(5)
    ref = rng.random((200_000, 3)).astype(np.float32)
    lay = oracle.build_tree(ref, 13)
    st, h = host_tree(ref, 13)
    check(st)
    try:
        pts, perm, med, off = layout_of(h, 200_000, 3, 13, np.float32)
    finally:
        LIB.tk_tree_destroy(h)
    np.testing.assert_array_equal(pts, lay.structured)
    np.testing.assert_array_equal(perm, lay.perm)
    np.testing.assert_array_equal(med, lay.medians)


def test_error_paths_without_gpu():
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL
    rng = np.random.default_rng(3)
    pts = rng.standard_normal((10, 3)).astype(np.float32)
    st, _ = host_tree(pts, 6)  # 32 split nodes for 10 points
    assert st == TK_EINVAL and "Ran out of points" in LIB.tk_last_error().decode()
    st, _ = host_tree(pts, 0)
    assert st == TK_EINVAL
    st, _ = host_tree(pts, 25)
    assert st == TK_EINVAL
    bad = pts.copy()
    bad[3, 1] = np.nan
    st, _ = host_tree(bad, 2)
    assert st == TK_EINVAL and "NaN" in LIB.tk_last_error().decode()
    nine_d = rng.standard_normal((10, 9)).astype(np.float32)
    st, _ = host_tree(nine_d, 2)  # KD trees go up to 8 dimensions
    assert st == TK_EINVAL
    # a host-only tree refuses queries instead of computing anything on the CPU
    st, h = host_tree(pts, 2)
    assert st == 0
    d = np.empty((1, 1), np.float32)
    i = np.empty((1, 1), np.int32)
    st = LIB.tk_tree_query(h, pts.ctypes.data, 1, 1, d.ctypes.data, i.ctypes.data, None, None, 0, None)
    assert st == TK_EINVAL
    LIB.tk_tree_destroy(h)


def test_misaligned_workspace_is_refused_before_device_work():
    """Workspaces are carved into 256-byte aligned sub-buffers (some read by bulk
    copies): a misaligned one fails with TK_EINVAL before anything touches a GPU."""
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL
    ref = np.zeros((100, 3), np.float32)
    q = np.zeros((10, 3), np.float32)
    d = np.empty((10, 2), np.float32)
    i = np.empty((10, 2), np.int32)
    g = np.zeros((10, 2), np.float32)
    ws = np.zeros(1 << 20, np.uint8)
    aligned = (ws.ctypes.data + 255) // 256 * 256
    for off in (4, 16, 128):
        st = LIB.tk_nn_distance(ref.ctypes.data, 100, q.ctypes.data, 10, 3, 2, 0, 0, d.ctypes.data, i.ctypes.data,
                                aligned + off, 1 << 19, None)
        assert st == TK_EINVAL and "256-byte aligned" in LIB.tk_last_error().decode()
        st = LIB.tk_knn_backward(q.ctypes.data, ref.ctypes.data, i.ctypes.data, g.ctypes.data, 10, 100, 2, 3, 0,
                                 None, ref.ctypes.data, aligned + off, 1 << 19, None)
        assert st == TK_EINVAL and "256-byte aligned" in LIB.tk_last_error().decode()


def test_default_levels_matches_reference_heuristic():
    from torch_kdtree_gb300 import default_levels
    for n, L in [(5, 1), (30, 1), (1000, 6), (100_000, 13), (4_194_304, 13), (16, 1), (128, 4)]:
        assert default_levels(n) == L


def tree_from_layout(pts, perm, med, off, levels, device=-1):
    from torch_kdtree_gb300._lib import LIB
    h = ctypes.c_void_p()
    dt = 0 if pts.dtype == np.float32 else 1
    st = LIB.tk_tree_create_from_layout(pts.ctypes.data, perm.ctypes.data, med.ctypes.data, off.ctypes.data,
                                        pts.shape[0], pts.shape[1], dt, levels, device, ctypes.byref(h))
    return st, h


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_layout_round_trip_and_validation(dtype, d):
    """A saved layout re-creates the same tree; corrupt layouts are refused
    (a tree whose splits do not separate its points would give inexact
    answers, so it must not load)."""
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL, check
    rng = np.random.default_rng(30 + d)
    ref = rng.standard_normal((3000, d)).astype(dtype)
    L = 7
    st, h = host_tree(ref, L)
    check(st)
    try:
        pts, perm, med, off = layout_of(h, 3000, d, L, ref.dtype)
    finally:
        LIB.tk_tree_destroy(h)
    st, h2 = tree_from_layout(pts, perm, med, off, L)
    check(st)
    try:
        again = layout_of(h2, 3000, d, L, ref.dtype)
    finally:
        LIB.tk_tree_destroy(h2)
    for a, b in zip((pts, perm, med, off), again):
        np.testing.assert_array_equal(a, b)

    def refused(p=pts, pe=perm, m=med, o=off, lv=L):
        st, hh = tree_from_layout(np.ascontiguousarray(p), np.ascontiguousarray(pe), np.ascontiguousarray(m),
                                  np.ascontiguousarray(o), lv)
        if hh.value:
            LIB.tk_tree_destroy(hh)
        return st == TK_EINVAL

    bad_perm = perm.copy()
    bad_perm[5] = bad_perm[6]
    assert refused(pe=bad_perm)
    bad_off = off.copy()
    bad_off[3] = bad_off[4] + 1  # decreasing offsets
    assert refused(o=bad_off)
    bad_end = off.copy()
    bad_end[-1] -= 1
    assert refused(o=bad_end)
    nan_pts = pts.copy()
    nan_pts[10, 0] = np.nan
    assert refused(p=nan_pts)
    moved = pts.copy()
    moved[0, 0] = med[0] + abs(med[0]) + 10  # first point belongs left of the root split along axis 0
    assert refused(p=moved)
    wrong_split = med.copy()
    wrong_split[0] = pts[:, 0].max() + 1
    assert refused(m=wrong_split)
    assert not refused(lv=L)


@pytest.mark.parametrize("device", ["cuda", "cpu"])
def test_uncompiled_dimension_raises_before_any_device_work(device):
    """The reference's test_uncompiled_dimension (tests/test_knn_unit.py:72-77):
    436 dimensions must raise, for either device string, before anything
    touches a GPU (KD trees take 1-8 dimensions, only CUDA trees exist, and a
    machine without a visible GPU refuses "cuda" up front)."""
    from torch_kdtree_gb300 import build_kd_tree
    with pytest.raises(Exception):
        build_kd_tree(np.random.uniform(size=(10, 436)), device=device)
