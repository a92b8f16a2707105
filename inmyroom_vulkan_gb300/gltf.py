"""glTF 2.0 meshes and scene instances as collision input.

The engine builds one OBB tree per glTF mesh from the triangles of its
primitives that are neither skinned nor morphed
(src/Graphics/Meshes/MeshesOfNodes.cpp:30-53,
src/Graphics/Meshes/PrimitivesOfMeshes.cpp:620-672, 835-862), each primitive's
index list expanded by its draw mode (CreateIndicesTriplets,
src/Geometry/Triangle.cpp:10-58; no index list: the vertices in order).
`load` reads a .gltf (with .bin buffers or data URIs) or a .glb into that
form: per mesh the concatenated points, normals and index triples of those
triangles, ready for `Context.build_trees`; and the scene's instances
(mesh, world matrix, column-major) by walking the node tree from the default
scene (TRS or matrix per node). `save` writes meshes and instances back as a
.gltf + .bin pair (triangle lists), for fixtures.

One difference from the engine: a triangle's stored vertex indices are the
mesh's (primitives' vertices concatenated), not the primitive's own; they
only key the deduplication of vertex rays. A primitive without normals in a
mesh whose other primitives have them gets its face normals
(TrianglePosition::GetTriangleFaceNormal, Triangle.cpp:140-146) on its own
copies of its corners.
"""
from __future__ import annotations

import base64
import json
import os
import struct
from dataclasses import dataclass, field

import numpy as np

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_COUNT = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
_TRIANGLES, _STRIP, _FAN = 4, 5, 6


@dataclass
class Mesh:
    name: str
    points: np.ndarray              # (V, 3) float32
    normals: np.ndarray | None      # (V, 3) float32 or None
    indices: np.ndarray             # (T, 3) uint32

    @property
    def n_tris(self) -> int:
        return len(self.indices)


@dataclass
class Instance:
    mesh: int
    matrix: np.ndarray              # (16,) float32, column-major world matrix
    node: str = ""


@dataclass
class Scene:
    meshes: list = field(default_factory=list)
    instances: list = field(default_factory=list)


def _buffers(doc: dict, base: str, glb_bin: bytes | None) -> list:
    out = []
    for b in doc.get("buffers", []):
        uri = b.get("uri")
        if uri is None:
            out.append(glb_bin or b"")
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            with open(os.path.join(base, uri), "rb") as f:
                out.append(f.read())
    return out


def _accessor(doc: dict, bufs: list, i: int) -> np.ndarray:
    a = doc["accessors"][i]
    dt = np.dtype(_COMPONENT[a["componentType"]])
    nc = _COUNT[a["type"]]
    count = a["count"]
    if "bufferView" not in a:
        return np.zeros((count, nc), dt)
    v = doc["bufferViews"][a["bufferView"]]
    raw = bufs[v["buffer"]]
    start = v.get("byteOffset", 0) + a.get("byteOffset", 0)
    stride = v.get("byteStride", 0) or dt.itemsize * nc
    if stride == dt.itemsize * nc:
        arr = np.frombuffer(raw, dt, count * nc, start).reshape(count, nc)
    else:
        arr = np.stack([np.frombuffer(raw, dt, nc, start + k * stride) for k in range(count)]) if count else \
            np.zeros((0, nc), dt)
    return arr.copy()


def triplets(indices: np.ndarray, mode: int) -> np.ndarray:
    """CreateIndicesTriplets (Triangle.cpp:10-58): the (T, 3) vertex triples
    a draw mode makes of an index list."""
    idx = np.asarray(indices, np.int64).reshape(-1)
    n = len(idx)
    if mode == _TRIANGLES:
        return idx[: 3 * (n // 3)].reshape(-1, 3)
    if mode == _STRIP:
        if n < 3:
            return np.zeros((0, 3), np.int64)
        i = np.arange(n - 2)
        return np.stack([idx[i], idx[i + 1 + i % 2], idx[i + 2 - i % 2]], 1)
    if mode == _FAN:
        if n < 3:
            return np.zeros((0, 3), np.int64)
        i = np.arange(n - 2)
        return np.stack([idx[i + 1], idx[i + 2], np.full(n - 2, idx[0])], 1)
    if mode == 0:  # points
        return np.stack([idx, idx, idx], 1)
    if mode == 1:  # lines
        m = n // 2
        return np.stack([idx[0:2 * m:2], idx[0:2 * m:2], idx[1:2 * m:2]], 1)
    if mode == 3:  # line strip
        if n < 2:
            return np.zeros((0, 3), np.int64)
        return np.stack([idx[:-1], idx[:-1], idx[1:]], 1)
    return np.zeros((0, 3), np.int64)  # line loop: no triangles in the engine either


def face_normals(p: np.ndarray) -> np.ndarray:
    """GetTriangleFaceNormal in float32 with the engine's operation order:
    normalize(cross(p1 - p0, p2 - p0)), normalize = v * (1 / sqrt(dot(v, v)))."""
    p = np.asarray(p, np.float32).reshape(-1, 3, 3)
    a = p[:, 1] - p[:, 0]
    b = p[:, 2] - p[:, 0]
    c = np.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                  a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], 1).astype(np.float32)
    d = (c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = (np.float32(1.0) / np.sqrt(d, dtype=np.float32)).astype(np.float32)
    return (c * inv[:, None]).astype(np.float32)


def _mesh(doc: dict, bufs: list, k: int) -> Mesh:
    m = doc["meshes"][k]
    parts = []
    for prim in m.get("primitives", []):
        attrs = prim.get("attributes", {})
        if "POSITION" not in attrs or "JOINTS_0" in attrs or "WEIGHTS_0" in attrs or prim.get("targets"):
            continue  # skinned or morphed primitives have no tree in the engine
        pos = _accessor(doc, bufs, attrs["POSITION"]).astype(np.float32)
        nrm = _accessor(doc, bufs, attrs["NORMAL"]).astype(np.float32) if "NORMAL" in attrs else None
        idx = (_accessor(doc, bufs, prim["indices"]).reshape(-1) if "indices" in prim
               else np.arange(len(pos)))
        parts.append((pos, nrm, triplets(idx, prim.get("mode", _TRIANGLES))))
    with_n = [p for p in parts if p[1] is not None]
    pts, nrms, tris, base = [], [], [], 0
    for pos, nrm, tri in parts:
        if with_n and nrm is None:  # mixed: this primitive's corners with their face normals
            corners = pos[tri.reshape(-1)]
            fn = face_normals(corners)
            pos, nrm = corners, np.repeat(fn, 3, axis=0)
            tri = np.arange(len(corners)).reshape(-1, 3)
        pts.append(pos)
        if with_n:
            nrms.append(nrm)
        tris.append(tri + base)
        base += len(pos)
    points = np.concatenate(pts) if pts else np.zeros((0, 3), np.float32)
    normals = np.concatenate(nrms).astype(np.float32) if with_n else None
    indices = (np.concatenate(tris) if tris else np.zeros((0, 3), np.int64)).astype(np.uint32)
    return Mesh(m.get("name", f"mesh{k}"), points.astype(np.float32), normals, indices)


def _node_matrix(n: dict) -> np.ndarray:
    if "matrix" in n:
        return np.asarray(n["matrix"], np.float64).reshape(4, 4).T  # stored column-major
    t = np.asarray(n.get("translation", [0, 0, 0]), np.float64)
    x, y, z, w = n.get("rotation", [0, 0, 0, 1])
    s = np.asarray(n.get("scale", [1, 1, 1]), np.float64)
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = r * s[None, :]
    M[:3, 3] = t
    return M


def load(path: str) -> Scene:
    """The meshes and instances of a .gltf or .glb file."""
    base = os.path.dirname(os.path.abspath(path))
    with open(path, "rb") as f:
        raw = f.read()
    glb_bin = None
    if raw[:4] == b"glTF":
        length = struct.unpack_from("<I", raw, 8)[0]
        off, doc = 12, None
        while off < length:
            clen, ctype = struct.unpack_from("<II", raw, off)
            chunk = raw[off + 8: off + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942:
                glb_bin = chunk
            off += 8 + clen
    else:
        doc = json.loads(raw.decode("utf-8"))
    bufs = _buffers(doc, base, glb_bin)
    out = Scene([_mesh(doc, bufs, k) for k in range(len(doc.get("meshes", [])))], [])
    nodes = doc.get("nodes", [])
    scenes = doc.get("scenes", [])
    roots = scenes[doc.get("scene", 0)]["nodes"] if scenes else list(range(len(nodes)))
    stack = [(r, np.eye(4)) for r in reversed(roots)]
    while stack:
        i, parent = stack.pop()
        n = nodes[i]
        world = parent @ _node_matrix(n)
        if "mesh" in n:
            out.instances.append(Instance(n["mesh"], world.T.reshape(16).astype(np.float32), n.get("name", "")))
        for c in reversed(n.get("children", [])):
            stack.append((c, world))
    return out


def save(path: str, scene: Scene) -> None:
    """`scene` as `path` (.gltf) and a .bin beside it: one triangle-list
    primitive per mesh (positions, normals when present, uint32 indices),
    one node per instance with its matrix."""
    blob = bytearray()
    views, accessors, meshes = [], [], []

    def add(arr: np.ndarray, ctype: int, typ: str, target: int) -> int:
        data = np.ascontiguousarray(arr).tobytes()
        while len(blob) % 4:
            blob.append(0)
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": len(data), "target": target})
        blob.extend(data)
        acc = {"bufferView": len(views) - 1, "componentType": ctype, "count": int(len(arr)), "type": typ}
        if typ == "VEC3" and len(arr):
            acc["min"] = [float(v) for v in np.asarray(arr).min(0)]
            acc["max"] = [float(v) for v in np.asarray(arr).max(0)]
        accessors.append(acc)
        return len(accessors) - 1

    for k, m in enumerate(scene.meshes):
        attrs = {"POSITION": add(np.asarray(m.points, np.float32).reshape(-1, 3), 5126, "VEC3", 34962)}
        if m.normals is not None:
            attrs["NORMAL"] = add(np.asarray(m.normals, np.float32).reshape(-1, 3), 5126, "VEC3", 34962)
        ind = add(np.asarray(m.indices, np.uint32).reshape(-1), 5125, "SCALAR", 34963)
        meshes.append({"name": m.name or f"mesh{k}", "primitives": [{"attributes": attrs, "indices": ind, "mode": 4}]})
    nodes = [{"mesh": int(inst.mesh), "matrix": [float(v) for v in np.asarray(inst.matrix, np.float32).reshape(16)],
              "name": inst.node} for inst in scene.instances]
    bin_name = os.path.splitext(os.path.basename(path))[0] + ".bin"
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": list(range(len(nodes)))}],
           "nodes": nodes, "meshes": meshes, "accessors": accessors, "bufferViews": views,
           "buffers": [{"uri": bin_name, "byteLength": len(blob)}]}
    with open(os.path.join(os.path.dirname(os.path.abspath(path)), bin_name), "wb") as f:
        f.write(bytes(blob))
    with open(path, "w") as f:
        json.dump(doc, f)
