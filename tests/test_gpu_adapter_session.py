"""The C++ adapters' core (adapter/cg_session.h: the calls GpuOBBtreesCollision
and GpuCreateUncollideRays make) in a C++ program on the GPU, against the
oracle: the candidate leaf pairs of ExecuteOBBtreesCollision and the rays and
mean origins of ExecuteCreateUncollideRays, bit for bit and in the
reference's order, for the 256-entity scene's AABB-overlap pairs. The engine
adapters themselves need the engine's headers and are compile-tested where
those are (test_adapter_compiles.py)."""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import build, scenes

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def write_input(path, meshes, qa, qb, mats):
    with open(path, "wb") as f:
        f.write(struct.pack("<I", len(meshes)))
        for m in meshes:
            pts = np.ascontiguousarray(m.points, np.float32).reshape(-1, 3)
            idx = np.ascontiguousarray(m.indices, np.uint32).reshape(-1)
            f.write(struct.pack("<III", len(pts), len(idx), 1 if m.normals is not None else 0))
            f.write(pts.tobytes())
            if m.normals is not None:
                f.write(np.ascontiguousarray(m.normals, np.float32).reshape(-1, 3).tobytes())
            f.write(idx.tobytes())
        f.write(struct.pack("<I", len(qa)))
        for a, b in zip(qa, qb):
            f.write(struct.pack("<II", int(a), int(b)))
            f.write(np.ascontiguousarray(mats[a], np.float32).tobytes())
            f.write(np.ascontiguousarray(mats[b], np.float32).tobytes())


def test_adapter_session_matches_oracle(tmp_path):
    lib = build.build()
    oracle.build_port()
    port_lib = os.path.join(build.ROOT, "oracle", "_build", "liboracle_port.so")
    exe = tmp_path / "adapter_session_check"
    cmd = ["g++", "-std=c++17", "-O2", "-I", build.INCLUDE, "-I", os.path.join(build.PKG, "adapter"),
           os.path.join(HERE, "adapter_session_check.cpp"), lib, port_lib, "-o", str(exe),
           f"-Wl,-rpath,{os.path.dirname(lib)}:{os.path.dirname(port_lib)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    sc = scenes.scene()
    inp = tmp_path / "scene.bin"
    write_input(inp, sc.meshes, sc.pairs[:, 0], sc.pairs[:, 1], sc.mats)
    r = subprocess.run([str(exe), str(inp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ok, nq, n_leaf, n_rays = r.stdout.split()
    assert ok == "ok" and int(nq) == len(sc.pairs) and int(n_leaf) > 100000 and int(n_rays) > 20000
