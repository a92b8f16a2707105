"""The C++ drop-in adapter compiles inside the engine's own sources: it is
built here against the reference's headers (with the glm shim standing in for
the absent glm submodule) and linked against libcollide_gpu.so and the
reference objects, without running (no GPU needed)."""
import os
import subprocess

import pytest

from inmyroom_vulkan_gb300 import build

from oracle import REF_ROOT_DEFAULT as REF
IMR = os.path.join(REF, "inMyRoom_vulkan")
ROOT = build.ROOT


@pytest.mark.skipif(not os.path.isdir(os.path.join(IMR, "include")), reason="reference sources not present")
def test_adapter_builds_against_reference_headers(tmp_path):
    lib = build.build()
    src = tmp_path / "use_adapter.cpp"
    src.write_text(
        '#include "gpu_obbtrees_collision.h"\n'
        "int main(int argc, char**) {\n"
        "    if (argc < 0) {  // never runs: this program only has to build and link\n"
        "        GpuOBBtreesCollision gpu;\n"
        "        GpuCreateUncollideRays rays(gpu.Shared());\n"
        "        std::pair<CollisionDetectionEntry, CollisionDetectionEntry> p{};\n"
        "        CDentriesPairTrianglesPairs r = gpu.ExecuteOBBtreesCollision(p);\n"
        "        CDentriesUncollideRays u = rays.ExecuteCreateUncollideRays(r);\n"
        "        return int(r.OBBtreesIntersectInfoObj.candidateTriangleRangeCombinations.size() +\n"
        "                   u.rays_from_first_to_second.size());\n"
        "    }\n"
        "    return 0;\n"
        "}\n")
    ref_lib = os.path.join(ROOT, "oracle", "_ref", "libimr_ref_strict.so")
    if not os.path.exists(ref_lib):
        import oracle

        oracle.build_ref()
    cmd = ["g++", "-std=c++20", "-O0", "-DENABLE_CPP_INTERFACE",
           "-I", os.path.join(ROOT, "oracle", "shim"), "-I", os.path.join(IMR, "include"),
           "-I", os.path.join(IMR, "shaders"), "-I", os.path.join(REF, "eig3"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "inmyroom_vulkan_gb300", "adapter"),
           str(src), ref_lib, lib, "-o", str(tmp_path / "use_adapter")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
