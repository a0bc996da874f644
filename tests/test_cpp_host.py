"""The C++ host interface (include/bhr_renderer.hpp): tests/cpp/renderer_tests.cpp compiled
against libbhr.so. Host checks run without a GPU; the traced frame is compared with the FP64
oracle and with the same view traced through the C ABI from Python, and its shaded image with
the CPU restatement of the shading; the frame traced through the learned surrogate under the
shader's rule (Settings::surrogate) is compared with the same-rule and converged FP64 oracles."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "renderer_tests.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "renderer_tests"
CUDA = Path("/usr/local/cuda")


def build() -> Path:
    from blackholerender_gb300._abi import LIB_PATH

    if not LIB_PATH.exists():
        pytest.skip("libbhr.so is not built")
    deps = [SRC, ROOT / "include" / "bhr_renderer.hpp", ROOT / "include" / "bhr.h", LIB_PATH]
    if EXE.exists() and EXE.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return EXE
    EXE.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}",
           str(SRC), "-o", str(EXE), f"-L{LIB_PATH.parent}", "-lbhr", f"-L{CUDA / 'lib64'}", "-lcudart",
           f"-Wl,-rpath,{LIB_PATH.parent}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    subprocess.run(cmd, check=True)
    return EXE


def test_cpp_host_checks():
    r = subprocess.run([str(build())], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " 0 failures" in r.stdout


@pytest.mark.gpu
def test_cpp_renderer_frame_vs_oracle(tmp_path):
    import parity
    from blackholerender_gb300 import HIT_DTYPE, TERM_CONFIG, Tracer, hits_numpy, workloads

    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT

    out = tmp_path / "frame.bin"
    r = subprocess.run([str(build()), "--gpu", str(out), "--surrogate", str(DEFAULT_CHECKPOINT)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    got = np.fromfile(out, dtype=HIT_DTYPE)
    v = workloads.c1_view(TERM_CONFIG)
    assert len(got) == v.rays
    with Tracer(0) as t:
        (o,) = t.trace([v])
        import torch

        torch.cuda.synchronize()
        direct = hits_numpy(o.cpu())
    assert np.array_equal(got.view(np.uint8), direct.view(np.uint8))  # same view, same kernel
    parity.check_fp32(got, v, where="C++ Renderer frame")
    # the image renderImage shaded from those records, against the CPU restatement of the shading
    import oracle_lib as O
    from blackholerender_gb300 import shade_params

    img = np.fromfile(str(out) + ".rgba", dtype=np.float32).reshape(v.height, v.width, 4)
    p = shade_params()
    ref = O.shade_view(v, got, p, O.noise_bake(p.noise_seed), O.blackbody_lut())
    d = np.abs(img - ref)
    assert np.mean(np.any(d > 1e-4 * np.abs(ref) + 1e-7, axis=-1)) <= 2e-3 and d.max() < 1e-3

    # the frame through the learned surrogate under the shader's rule (480x270, High preset,
    # thin disk, the same camera): the records of bhr_trace with the surrogate bound, and the
    # surrogate path's bars against the same-rule and the converged FP64 oracles
    import math

    from blackholerender_gb300 import METHOD_SURROGATE, TERM_SHADER, make_view
    from blackholerender_gb300.surrogate import DEFAULT_CHECKPOINT, Surrogate

    sv = make_view(TERM_SHADER, width=480, height=270, fov_deg=60.0, preset=2, pose=(30.0, math.radians(85.0), 0.0))
    gs = np.fromfile(str(out) + ".surrogate", dtype=HIT_DTYPE)
    assert len(gs) == sv.rays
    s = Surrogate(seed=1)
    s.load(str(DEFAULT_CHECKPOINT))
    with Tracer(0) as t:
        t.set_surrogate(s)
        (o,) = t.trace([sv], method=METHOD_SURROGATE)
        torch.cuda.synchronize()
        assert np.array_equal(gs.view(np.uint8), hits_numpy(o.cpu()).view(np.uint8))
        t.set_surrogate(None)
    s.close()
    idx = np.random.default_rng(3).choice(sv.rays, 3000, replace=False)
    print(parity.check_surrogate(gs, sv, idx, where="C++ Renderer surrogate frame"))
