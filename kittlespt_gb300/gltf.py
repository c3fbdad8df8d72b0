"""glTF 2.0 scene files (.gltf with external or embedded buffers, .glb) into a
Scene, following the reference SampleApp's importer
(SampleApp/src/sample_app/model_importer.hpp:51-456):

* the top-level nodes of scenes[0] (their children are not visited, as in the
  reference, :434-455); a node with a mesh becomes one mesh and one instance
  with the node's matrix, or T * R * S from its translation, rotation
  (quaternion x, y, z, w) and scale (:144-222); the first node with a camera
  becomes the camera: view = inverse(T * R(normalised)) and the vertical
  field of view (:380-432), converted the way Renderer::loadScene converts a
  CameraSceneEntity (renderer.cu:420-430: inverse view with its third column
  negated, the inverse of a left-handed perspective of that field of view,
  aspect 1, near 1, far 100);
* triangles are the primitives' indexed POSITION / NORMAL / TEXCOORD_0, one
  material per primitive (:224-276);
* images are decoded to 8-bit RGB, as stbi_load(..., 3) gives them (:278-317);
  PNG only here (8-bit, non-interlaced, any colour type), JPEG is refused;
* materials (:319-377): baseColorFactor rgb and baseColorTexture,
  metallicFactor / roughnessFactor and metallicRoughnessTexture,
  normalTexture and its scale, emissiveFactor and emissiveTexture, and the
  extensions KHR_materials_transmission (factor, texture), KHR_materials_ior
  (default 1.45) and KHR_materials_emissive_strength (default 0: without it
  nothing emits, as in the reference).  Texture references are image
  indices (textures[i].source).

Beyond the reference (which reads only unsigned-short indices from buffer 0
and ignores accessor offsets and strides): any unsigned index type, accessor
and view offsets, strides, data: URIs, non-indexed primitives, a missing
NORMAL (flat normals) or TEXCOORD_0 (zeros), and primitives without a
material (the glTF default material, appended)."""

from __future__ import annotations

import base64
import json
import math
import os
import struct
import zlib
from typing import List, Optional

import numpy as np

from . import scenes as S

_COMPONENTS = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_WIDTH = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


# --------------------------------------------------------------------------- files

def _read(path):
    with open(path, "rb") as f:
        data = f.read()
    base = os.path.dirname(os.path.abspath(path))
    if data[:4] == b"glTF":
        version, length = struct.unpack_from("<II", data, 4)
        if version != 2:
            raise ValueError(f"{path}: glTF version {version} (2 is supported)")
        off, doc, bin_chunk = 12, None, None
        while off < length:
            clen, ctype = struct.unpack_from("<II", data, off)
            chunk = data[off + 8:off + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942:
                bin_chunk = chunk
            off += 8 + clen
        if doc is None:
            raise ValueError(f"{path}: no JSON chunk")
    else:
        doc, bin_chunk = json.loads(data.decode("utf-8")), None
    buffers = []
    for k, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if bin_chunk is None:
                raise ValueError(f"{path}: buffer {k} has no data")
            buffers.append(bin_chunk)
        elif uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            with open(os.path.join(base, uri), "rb") as f:
                buffers.append(f.read())
    return doc, buffers, base


def _view_bytes(doc, buffers, view_index):
    v = doc["bufferViews"][view_index]
    b = buffers[v["buffer"]]
    off = v.get("byteOffset", 0)
    return b[off:off + v["byteLength"]], v.get("byteStride", 0)


def _accessor(doc, buffers, index):
    a = doc["accessors"][index]
    dt = np.dtype(_COMPONENTS[a["componentType"]]).newbyteorder("<")
    width = _WIDTH[a["type"]]
    count = a["count"]
    if "bufferView" not in a:
        return np.zeros((count, width), dt)
    raw, stride = _view_bytes(doc, buffers, a["bufferView"])
    off = a.get("byteOffset", 0)
    elem = dt.itemsize * width
    stride = stride or elem
    buf = np.frombuffer(raw, np.uint8)
    rows = np.stack([buf[off + i * stride:off + i * stride + elem] for i in range(count)]) if stride != elem else \
        buf[off:off + count * elem].reshape(count, elem)
    out = np.ascontiguousarray(rows).view(dt).reshape(count, width)
    if a.get("normalized") and dt.kind in "iu":
        out = out.astype(np.float32) / np.float32(np.iinfo(dt).max)
    return out


# --------------------------------------------------------------------------- PNG

def _png_rgb(data: bytes) -> np.ndarray:
    """8-bit non-interlaced PNG to [h, w, 3] uint8 (grey replicated, alpha
    dropped, palettes expanded), as stbi_load with 3 requested channels."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        if data[:2] == b"\xff\xd8":
            raise ValueError("JPEG textures are not supported: convert them to PNG")
        raise ValueError("unknown image format")
    off, idat, plte = 8, [], None
    w = h = depth = ctype = interlace = None
    while off < len(data):
        n, = struct.unpack_from(">I", data, off)
        kind = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        off += 12 + n
    if depth != 8 or interlace != 0:
        raise ValueError("PNG textures must be 8-bit and non-interlaced")
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, 1 + w * ch)
    img = np.zeros((h, w * ch), np.int32)
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        cur = np.zeros(w * ch, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for i in range(w * ch):
                a = cur[i - ch] if i >= ch else 0
                b = prev[i]
                c = prev[i - ch] if i >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[i] = (line[i] + p) & 255
        img[y] = cur
        prev = cur
    img = img.astype(np.uint8).reshape(h, w, ch)
    if ctype == 3:
        return plte[img[..., 0]]
    if ch in (1, 2):
        return np.repeat(img[..., :1], 3, axis=2)
    return np.ascontiguousarray(img[..., :3])


# --------------------------------------------------------------------------- scene

def _quat(q):   # glm::toMat4 of quat(w, x, y, z)
    x, y, z, w = (float(v) for v in q)
    m = np.eye(4)
    m[0, 0] = 1 - 2 * (y * y + z * z); m[0, 1] = 2 * (x * y - w * z); m[0, 2] = 2 * (x * z + w * y)
    m[1, 0] = 2 * (x * y + w * z); m[1, 1] = 1 - 2 * (x * x + z * z); m[1, 2] = 2 * (y * z - w * x)
    m[2, 0] = 2 * (x * z - w * y); m[2, 1] = 2 * (y * z + w * x); m[2, 2] = 1 - 2 * (x * x + y * y)
    return m


def _node_matrix(node, normalise_rotation=False, with_scale=True):
    if "matrix" in node:
        return np.asarray(node["matrix"], float).reshape(4, 4).T
    t = S.translate(*node.get("translation", (0.0, 0.0, 0.0)))
    r = np.eye(4)
    if "rotation" in node:
        q = np.asarray(node["rotation"], float)
        if normalise_rotation:
            q = q / np.linalg.norm(q)
        r = _quat(q)
    s = np.eye(4)
    if with_scale and "scale" in node:
        s[0, 0], s[1, 1], s[2, 2] = node["scale"]
    return t @ r @ s


def _material(doc, m):
    def source(info):
        return doc["textures"][info["index"]]["source"] if info is not None and info.get("index", -1) >= 0 else -1
    pbr = m.get("pbrMetallicRoughness", {})
    ext = m.get("extensions", {})
    rec = S.material(albedo=tuple(pbr.get("baseColorFactor", (1, 1, 1, 1))[:3]),
                     metallic=pbr.get("metallicFactor", 1.0), roughness=pbr.get("roughnessFactor", 1.0),
                     transmission=ext.get("KHR_materials_transmission", {}).get("transmissionFactor", 0.0),
                     ior=ext.get("KHR_materials_ior", {}).get("ior", 1.45),
                     emission=tuple(m.get("emissiveFactor", (0, 0, 0))),
                     emission_scale=ext.get("KHR_materials_emissive_strength", {}).get("emissiveStrength", 0.0))
    rec["albedo_tex"] = source(pbr.get("baseColorTexture"))
    rec["orm_tex"] = source(pbr.get("metallicRoughnessTexture"))
    rec["normal_tex"] = source(m.get("normalTexture"))
    rec["normal_scale"] = (m.get("normalTexture") or {}).get("scale", 1.0)
    rec["emission_tex"] = source(m.get("emissiveTexture"))
    rec["transmission_tex"] = source(ext.get("KHR_materials_transmission", {}).get("transmissionTexture"))
    return rec


def _mesh(doc, buffers, mesh, default_material):
    pos, nrm, uv, mat = [], [], [], []
    for prim in mesh["primitives"]:
        if prim.get("mode", 4) != 4:
            raise ValueError(f"mesh {mesh.get('name', '')}: only triangle primitives are supported")
        attr = prim["attributes"]
        p = _accessor(doc, buffers, attr["POSITION"]).astype(np.float32)
        idx = (_accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.int64) if "indices" in prim
               else np.arange(p.shape[0]))
        tp = p[idx].reshape(-1, 3, 3)
        if "NORMAL" in attr:
            tn = _accessor(doc, buffers, attr["NORMAL"]).astype(np.float32)[idx].reshape(-1, 3, 3)
        else:
            g = np.cross(tp[:, 1] - tp[:, 0], tp[:, 2] - tp[:, 0]).astype(np.float64)
            g /= np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-30)
            tn = np.repeat(g[:, None, :], 3, axis=1).astype(np.float32)
        if "TEXCOORD_0" in attr:
            tu = _accessor(doc, buffers, attr["TEXCOORD_0"]).astype(np.float32)[idx].reshape(-1, 3, 2)
        else:
            tu = np.zeros((tp.shape[0], 3, 2), np.float32)
        m = prim.get("material", -1)
        pos.append(tp)
        nrm.append(tn)
        uv.append(tu)
        mat.append(np.full(tp.shape[0], m if m >= 0 else default_material, np.int32))
    return S.Mesh(np.ascontiguousarray(np.concatenate(pos), np.float32),
                  np.ascontiguousarray(np.concatenate(nrm), np.float32),
                  np.ascontiguousarray(np.concatenate(uv), np.float32), np.concatenate(mat))


def camera_from_view(view, yfov):
    """Renderer::loadScene's camera from a CameraSceneEntity (renderer.cu:420-
    430): the inverse view with its third column negated, the inverse of a
    left-handed perspective of yfov at aspect 1 (near 1, far 100)."""
    inv_view = np.linalg.inv(np.asarray(view, float))
    inv_view[:, 2] *= -1.0
    inv_proj = np.linalg.inv(S.perspective_fov_lh(yfov, 100.0, 100.0, 1.0, 100.0))
    return S.Camera(inv_proj.astype(np.float32), inv_view.astype(np.float32))


def load_gltf(path, width=256, height=256, spp=1, max_depth=3, camera: Optional[S.Camera] = None) -> S.Scene:
    """The scene of a .gltf / .glb file.  `camera` replaces (or, when the file
    has none, supplies) the camera."""
    doc, buffers, base = _read(path)
    textures: List[np.ndarray] = []
    for img in doc.get("images", []):
        if "bufferView" in img:
            data, _ = _view_bytes(doc, buffers, img["bufferView"])
        elif img.get("uri", "").startswith("data:"):
            data = base64.b64decode(img["uri"].split(",", 1)[1])
        else:
            with open(os.path.join(base, img["uri"]), "rb") as f:
                data = f.read()
        textures.append(_png_rgb(bytes(data)))
    mats = [_material(doc, m) for m in doc.get("materials", [])]
    default_material = len(mats)
    mats.append(S.material(albedo=(1.0, 1.0, 1.0), metallic=1.0, roughness=1.0, emission_scale=0.0))
    meshes, instances, cam = [], [], None
    for ni in doc["scenes"][0]["nodes"]:
        node = doc["nodes"][ni]
        if node.get("camera", -1) >= 0 and cam is None:
            c = doc["cameras"][node["camera"]]
            model = _node_matrix(node, normalise_rotation=True, with_scale=False)
            cam = camera_from_view(np.linalg.inv(model), float(c["perspective"]["yfov"]))
        if node.get("mesh", -1) >= 0:
            meshes.append(_mesh(doc, buffers, doc["meshes"][node["mesh"]], default_material))
            instances.append(S.Instance(len(meshes) - 1, _node_matrix(node).astype(np.float32), -1))
    if camera is not None:
        cam = camera
    if cam is None:
        raise ValueError(f"{path}: no camera node; pass camera=")
    if not meshes:
        raise ValueError(f"{path}: no mesh nodes in scenes[0]")
    return S.Scene(meshes=meshes, instances=instances, materials=np.stack(mats), camera=cam,
                   env=S.environment(), settings=S.settings(max_depth=max_depth), exposure=S.exposure(),
                   width=width, height=height, spp=spp, name=os.path.basename(path), textures=textures)
