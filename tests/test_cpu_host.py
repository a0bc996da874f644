"""Host logic without a GPU: the C ABI library loads and exports every entry point bhr.h
declares with the layouts the Python mirror assumes; view helpers; the seeded workloads
against libstdc++'s own generator; sharding across two gloo ranks."""
from __future__ import annotations

import ctypes
import math
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from blackholerender_gb300 import _abi, make_view, workloads
from blackholerender_gb300.sharding import partition_views, view_cost

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "bhr.h"


def declared_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w \*]*?\b(bhr_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) >= 40
    L = _abi.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing
    assert sorted(_abi.SIGNATURES) == names  # the Python mirror binds exactly the header's functions
    assert L.bhr_abi_version() == 1


def test_struct_layouts_match_the_header(tmp_path):
    src = tmp_path / "layout.c"
    fields = {
        "bhr_view": [f for f, _ in _abi.View._fields_],
        "bhr_options": [f for f, _ in _abi.Options._fields_],
        "bhr_stats": [f for f, _ in _abi.Stats._fields_],
        "bhr_launch_shape": [f for f, _ in _abi.LaunchShape._fields_],
        "bhr_surrogate_config": [f for f, _ in _abi.SurrogateConfig._fields_],
        "bhr_shade_params": [f for f, _ in _abi.ShadeParams._fields_],
        "bhr_body": [f for f, _ in _abi.Body._fields_],
        "bhr_body_hit": list(_abi.BODY_HIT_DTYPE.names),
        "bhr_hit": list(_abi.HIT_DTYPE.names),
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bhr.h"', "int main(void) {"]
    for st, fs in fields.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fs:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True)
               .stdout.splitlines())
    py = {"bhr_view": _abi.View, "bhr_options": _abi.Options, "bhr_stats": _abi.Stats,
          "bhr_launch_shape": _abi.LaunchShape, "bhr_surrogate_config": _abi.SurrogateConfig,
          "bhr_shade_params": _abi.ShadeParams, "bhr_body": _abi.Body}
    for st, cls in py.items():
        assert int(got[st]) == ctypes.sizeof(cls), st
        for f, _ in cls._fields_:
            assert int(got[f"{st}.{f}"]) == getattr(cls, f).offset, (st, f)
    assert int(got["bhr_body_hit"]) == _abi.BODY_HIT_DTYPE.itemsize == 64
    for f in _abi.BODY_HIT_DTYPE.names:
        assert int(got[f"bhr_body_hit.{f}"]) == _abi.BODY_HIT_DTYPE.fields[f][1], f
    assert int(got["bhr_hit"]) == _abi.HIT_DTYPE.itemsize == 64
    for f in _abi.HIT_DTYPE.names:
        assert int(got[f"bhr_hit.{f}"]) == _abi.HIT_DTYPE.fields[f][1], f


def test_create_without_a_device_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    ctx = ctypes.c_void_p()
    rc = _abi.lib().bhr_create(ctypes.byref(ctx), None)
    assert rc == _abi.ERR_CUDA and not ctx
    assert b"no CUDA device" in _abi.lib().bhr_last_error(None)


def test_view_defaults_and_presets():
    v = make_view(_abi.TERM_SHADER)
    assert (v.width, v.height, v.max_steps) == (1920, 1080, 450)
    assert (v.step_scale, v.disk_step) == (np.float32(0.05), np.float32(0.18))
    assert (v.disk_inner, v.disk_outer) == (6.0, 20.0) and abs(v.disk_thickness - 0.035) < 1e-7
    assert abs(v.capture_r - 2.02) < 1e-6 and v.r_esc_min == 25.0 and abs(v.ds_floor - 0.02) < 1e-7
    assert abs(v.tan_half_fov - math.tan(math.radians(30.0))) < 1e-7
    for p, (ms, ss, ds) in enumerate([(200, 0.10, 0.35), (300, 0.07, 0.30), (450, 0.05, 0.18), (700, 0.035, 0.10)]):
        w = make_view(_abi.TERM_CONFIG, preset=p)
        assert w.max_steps == ms and abs(w.step_scale - ss) < 1e-7 and abs(w.disk_step - ds) < 1e-7
    c = make_view(_abi.TERM_CPU)
    assert c.max_steps == 200000 and abs(c.capture_r - 2.01) < 1e-6 and c.disk_mode == _abi.DISK_NONE
    with pytest.raises(_abi.BhrError):
        make_view(_abi.TERM_SHADER, preset=7)


def test_orbit_pose_looks_at_the_hole():
    r, inc, az = 33.0, math.radians(70.0), 1.2
    v = make_view(_abi.TERM_CONFIG, pose=(r, inc, az))
    pos = np.array(v.cam_pos[:], dtype=np.float64)
    want = r * np.array([math.sin(inc) * math.sin(az), math.cos(inc), math.sin(inc) * math.cos(az)])
    assert np.allclose(pos, want, rtol=1e-6)
    B = np.array(v.cam_basis[:], dtype=np.float64).reshape(3, 3)  # rows = columns right, up, back
    assert np.allclose(B @ B.T, np.eye(3), atol=1e-6)
    assert np.dot(B[2], pos / np.linalg.norm(pos)) > 1 - 1e-6  # back column away from the hole
    assert abs(B[0][1]) < 1e-6  # roll 0


def test_mt19937_64_known_answer():
    # C++ [rand.predef]: the 10000th output of a default-constructed std::mt19937_64
    g = workloads.MT19937_64(5489)
    x = 0
    for _ in range(10000):
        x = g()
    assert x == 9981545732273789042


def test_poses_match_libstdcxx(tmp_path):
    """The 16 poses of the 1080p configuration, drawn as std::mt19937_64(0) with
    std::uniform_real_distribution<double> (r, inclination, azimuth per pose)."""
    src = tmp_path / "poses.cpp"
    src.write_text(r'''
#include <cmath>
#include <cstdio>
#include <random>
int main() {
    std::mt19937_64 g(0);
    std::uniform_real_distribution<double> R(15.0, 60.0), I(60.0 * M_PI / 180.0, 90.0 * M_PI / 180.0), A(0.0, 2.0 * M_PI);
    for (int k = 0; k < 16; ++k) { double r = R(g), i = I(g), a = A(g); std::printf("%.17g %.17g %.17g\n", r, i, a); }
}''')
    exe = tmp_path / "poses"
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-o", str(exe)], check=True)
    ref = np.loadtxt(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    got = np.array(workloads.c2_poses())
    assert np.array_equal(got, ref)


def test_oracle_builds_the_same_views_as_the_library():
    """The CPU arm of the benchmark builds its views with the oracle alone (no product library
    mapped); those views must be the library's to the byte: C1, the 16 C2 poses under both
    rules, the 64 C4 views, and an inclination below the lookRotation up-vector fallback."""
    import oracle_lib as O

    cases = [(_abi.TERM_CONFIG, 0, 256, 144, 60.0, (30.0, math.radians(85.0), 0.0)),
             (_abi.TERM_SHADER, 3, 640, 360, 40.0, (20.0, math.radians(88.0), 0.0)),
             (_abi.TERM_CPU, -1, 64, 36, 75.0, (40.0, math.radians(1.0), 0.3))]
    for term in (_abi.TERM_CONFIG, _abi.TERM_SHADER):
        cases += [(term, 2, 1920, 1080, 60.0, p) for p in workloads.c2_poses()]
    cases += [(_abi.TERM_CONFIG, pre, w, h, fov, pose) for w, h, fov, pre, pose in workloads.c4_specs()]
    for term, pre, w, h, fov, pose in cases:
        a = O.orbit_view(term, pre, w, h, fov, pose)
        b = make_view(term, width=w, height=h, fov_deg=fov, preset=None if pre < 0 else pre, pose=pose)
        assert bytes(a) == bytes(b), (term, pre, w, h, fov, pose)


def test_partition_is_balanced_and_complete():
    views = workloads.c4_views(_abi.TERM_CONFIG, scale=0.05)
    for world in (1, 2, 4, 8):
        parts = partition_views(views, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(views)))
        loads = [sum(view_cost(views[k]) for k in p) for p in parts]
        biggest = max(view_cost(v) for v in views)
        assert max(loads) - min(loads) <= biggest + 1e-6
        assert partition_views(views, world) == parts  # deterministic


def _shard_worker(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import oracle_lib as O
    from blackholerender_gb300.sharding import gather_records

    dist.init_process_group("gloo", rank=rank, world_size=world)
    views = workloads.c4_views(_abi.TERM_CONFIG, scale=0.0005, n=10)
    mine = partition_views(views, world)[rank]
    # the per-rank compute is stood in for by the CPU oracle; the sharding logic is what is tested
    local = {k: O.trace_view(views[k], fp64=True, threads=2) for k in mine}
    got = gather_records(local, views, world, rank)
    if rank == 0:
        np.save(out_dir / "gathered.npy", np.concatenate([g.view(np.uint8) for g in got]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_gathers_every_view(tmp_path):
    import sys

    import torch.multiprocessing as mp

    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O

    port = 29500 + os.getpid() % 1000
    mp.start_processes(_shard_worker, args=(2, port, tmp_path), nprocs=2, start_method="spawn")
    views = workloads.c4_views(_abi.TERM_CONFIG, scale=0.0005, n=10)
    want = np.concatenate([O.trace_view(v, fp64=True, threads=2).view(np.uint8) for v in views])
    assert np.array_equal(np.load(tmp_path / "gathered.npy"), want)
