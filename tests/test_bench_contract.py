"""Host-side pieces of bench.py that need no GPU: the roofline inputs read
from the committed ncu summaries, and the algorithmic byte count."""
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_roofline_inputs_come_from_the_committed_profile():
    b = bench()
    tag = "kd_query_cube_sphere_4M_k16"
    traffic = b.profiled_traffic(tag)
    inst = b.profiled_value(tag, "warp_instructions_per_launch")
    assert isinstance(traffic, int) and traffic > 100_000_000
    assert isinstance(inst, int) and inst > 1_000_000_000
    assert b.profiled_traffic("no_such_profile") is None
    # the batched row's DRAM traffic: one launch over the 256 ragged clouds
    batch = b.profiled_traffic("batch_query_256_ragged")
    assert isinstance(batch, int) and 400_000_000 < batch < 2_000_000_000


def test_algorithmic_bytes_of_the_headline_launch():
    b = bench()
    # 1,048,576 queries x (12 B in + 128 B out) + 4,194,304 points x 12 B + 8 B per split node at depth 18
    got = b.algorithmic_bytes(4_194_304, 1_048_576, 16, 18)
    assert got == 1_048_576 * 140 + 4_194_304 * 12 + 8 * ((1 << 18) - 1)
    assert 199e6 < got < 200e6
    # the same in this engine's layout: 16-byte records, 4-byte splits and leaf offsets
    lay = b.layout_bytes(4_194_304, 1_048_576, 16, 18)
    assert lay == 1_048_576 * 140 + 4_194_304 * 16 + 4 * ((1 << 18) - 1) + 4 * ((1 << 18) + 1)


def test_profile_figures_only_for_the_profiled_launch_shape(tmp_path, monkeypatch):
    b = bench()
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "kd_query_x.md").write_text("profiled_shape: " + b.launch_shape(18, 1, 1) + "\n"
                                        "traffic_bytes_per_launch: 123\nwarp_instructions_per_launch: 456\n")
    monkeypatch.setattr(b, "ROOT", str(tmp_path))
    assert b.profiled_traffic("kd_query_x", b.launch_shape(18, 1, 1)) == 123
    assert b.profiled_traffic("kd_query_x", b.launch_shape(17, 1, 1)) is None
    assert b.profiled_value("kd_query_x", "warp_instructions_per_launch", b.launch_shape(18, 1, 1)) == 456
    assert b.profiled_traffic("kd_query_x") == 123


def test_every_profile_names_its_command():
    for f in sorted(os.listdir(os.path.join(ROOT, "profiles"))):
        text = open(os.path.join(ROOT, "profiles", f)).read()
        assert f.endswith(".md")
        assert "python bench.py" in text and "--clock-control none" in text, f


def test_reference_arm_maps_no_library_of_this_package():
    """`bench.py --impl reference` times the reference's CPU query path; it
    must not import this package or map its CUDA library (only the
    oracle's libraries), so the two arms stay separate programs."""
    import subprocess
    import sys
    code = (
        "import importlib.util, os, sys, types\n"
        f"root = {ROOT!r}\n"
        "sys.path.insert(0, root)\n"
        "spec = importlib.util.spec_from_file_location('bench_mod', os.path.join(root, 'bench.py'))\n"
        "b = importlib.util.module_from_spec(spec); spec.loader.exec_module(b)\n"
        "b.run_reference(types.SimpleNamespace(ref_sample=512, steps=1, warmup=0, gpus=1))\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libtkknn' not in maps, 'the reference arm mapped libtkknn.so'\n"
        "bad = [m for m in sys.modules if m.startswith('torch_kdtree_gb300')]\n"
        "assert not bad, bad\n"
        "assert 'liboracle' in maps or 'libtkref' in maps\n"
        "print('REFERENCE_ARM_OK')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "REFERENCE_ARM_OK" in r.stdout
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["impl"] == "reference" and line["e2e"]["h2d_bytes_per_step"] == 0
