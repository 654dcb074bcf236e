"""Writes glTF 2.0 files for the scene-ingestion tests: one binary buffer holding every accessor,
saved as an external .bin, a base64 data URI or a .glb container."""
from __future__ import annotations

import base64
import json
import struct

import numpy as np

COMPONENT = {np.dtype(np.int8): 5120, np.dtype(np.uint8): 5121, np.dtype(np.int16): 5122,
             np.dtype(np.uint16): 5123, np.dtype(np.uint32): 5125, np.dtype(np.float32): 5126}
TYPE = {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4"}


class GltfBuilder:
    def __init__(self):
        self.blob = bytearray()
        self.j = {"asset": {"version": "2.0", "generator": "gbpt tests"}, "buffers": [], "bufferViews": [],
                  "accessors": [], "meshes": [], "nodes": [], "materials": [], "cameras": [],
                  "scenes": [{"nodes": []}], "scene": 0}

    def accessor(self, array, stride: int | None = None, extra: dict | None = None) -> int:
        """Appends array (N, width) or (N,) as one bufferView (interleaved with padding when stride is
        larger than an element) and returns its accessor index."""
        a = np.asarray(array)
        a2 = a.reshape(len(a), -1)
        width = a2.shape[1]
        elem = a2.dtype.itemsize * width
        while len(self.blob) % 4:
            self.blob.append(0)
        start = len(self.blob)
        if stride is None or stride == elem:
            self.blob += a2.astype(a2.dtype.newbyteorder("<")).tobytes()
            view = {"buffer": 0, "byteOffset": start, "byteLength": len(self.blob) - start}
        else:
            for row in a2:
                chunk = row.astype(a2.dtype.newbyteorder("<")).tobytes()
                self.blob += chunk + b"\xAB" * (stride - len(chunk))
            view = {"buffer": 0, "byteOffset": start, "byteLength": len(self.blob) - start, "byteStride": stride}
        self.j["bufferViews"].append(view)
        acc = {"bufferView": len(self.j["bufferViews"]) - 1, "componentType": COMPONENT[a2.dtype],
               "count": len(a2), "type": TYPE[width]}
        if extra:
            acc.update(extra)
        self.j["accessors"].append(acc)
        return len(self.j["accessors"]) - 1

    def mesh(self, primitives) -> int:
        self.j["meshes"].append({"primitives": primitives})
        return len(self.j["meshes"]) - 1

    def node(self, root: bool = True, **fields) -> int:
        self.j["nodes"].append(fields)
        i = len(self.j["nodes"]) - 1
        if root:
            self.j["scenes"][0]["nodes"].append(i)
        return i

    def save(self, path: str, container: str = "file") -> str:
        """container: 'file' (path + '.gltf' beside path + '.bin'), 'base64' (one .gltf) or 'glb'."""
        j = json.loads(json.dumps(self.j))
        for k in ("materials", "cameras", "meshes"):
            if not j[k]:
                del j[k]
        blob = bytes(self.blob)
        if container == "glb":
            j["buffers"] = [{"byteLength": len(blob)}]
            text = json.dumps(j).encode()
            text += b" " * (-len(text) % 4)
            body = blob + b"\0" * (-len(blob) % 4)
            out = path + ".glb"
            total = 12 + 8 + len(text) + 8 + len(body)
            with open(out, "wb") as f:
                f.write(struct.pack("<4sII", b"glTF", 2, total))
                f.write(struct.pack("<II", len(text), 0x4E4F534A) + text)
                f.write(struct.pack("<II", len(body), 0x004E4942) + body)
            return out
        out = path + ".gltf"
        if container == "base64":
            j["buffers"] = [{"byteLength": len(blob),
                             "uri": "data:application/octet-stream;base64," + base64.b64encode(blob).decode()}]
        else:
            name = path.rsplit("/", 1)[-1] + " data.bin"  # a space: the URI is percent-encoded
            with open(path.rsplit("/", 1)[0] + "/" + name, "wb") as f:
                f.write(blob)
            j["buffers"] = [{"byteLength": len(blob), "uri": name.replace(" ", "%20")}]
        with open(out, "w") as f:
            json.dump(j, f, indent=1)
        return out


def scene_file(path: str, positions, indices, material_of, materials, camera=None, container="file") -> str:
    """A flat scene (one node, one primitive per material) written as glTF: the identity transform
    keeps every position bit-exact through the loader."""
    b = GltfBuilder()
    b.j["materials"] = list(materials)
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.asarray(indices, np.int64).reshape(-1, 3)
    mat = np.asarray(material_of)
    pacc = b.accessor(pos)
    prims = []
    for m in range(len(materials)):
        tri = idx[mat == m]
        if len(tri):
            prims.append({"attributes": {"POSITION": pacc}, "indices": b.accessor(tri.reshape(-1).astype(np.uint32)),
                          "material": m})
    b.node(mesh=b.mesh(prims))
    if camera is not None:
        b.j["cameras"].append({"type": "perspective", "perspective": camera["perspective"]})
        b.node(camera=0, **camera.get("transform", {}))
    return b.save(path, container)
