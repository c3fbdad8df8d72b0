"""glTF ingestion (kittlespt_gb300/gltf.py, after the reference SampleApp's
importer): PNG decoding, accessor reading, the node / material / camera
mapping, .gltf and .glb giving the same scene, and -- on the GPU -- a
textured glTF scene rendered against the oracle."""

import base64
import json
import math
import os
import struct
import zlib

import numpy as np
import pytest

from kittlespt_gb300 import gltf as G
from kittlespt_gb300 import scenes as S


def _png(img, filters=(0, 1, 2, 3, 4), ctype=None, palette=None):
    """A PNG of img ([h, w, c] uint8), each row with the next filter of `filters`."""
    h, w = img.shape[:2]
    ch = img.shape[2]
    ctype = ctype if ctype is not None else {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    rows, prev = [], np.zeros(w * ch, np.int32)
    for y in range(h):
        line = img[y].reshape(-1).astype(np.int32)
        f = filters[y % len(filters)]
        out = np.zeros_like(line)
        for i in range(w * ch):
            a = line[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            p = {0: 0, 1: a, 2: b, 3: (a + b) >> 1}.get(f)
            if f == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            out[i] = (line[i] - p) & 255
        rows.append(bytes([f]) + out.astype(np.uint8).tobytes())
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    return data + chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b"")


def test_png_decoding():
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (7, 9, 3), np.uint8)
    assert np.array_equal(G._png_rgb(_png(rgb)), rgb)
    rgba = rng.integers(0, 256, (5, 6, 4), np.uint8)
    assert np.array_equal(G._png_rgb(_png(rgba)), rgba[..., :3])
    grey = rng.integers(0, 256, (4, 5, 1), np.uint8)
    assert np.array_equal(G._png_rgb(_png(grey)), np.repeat(grey, 3, axis=2))
    pal = rng.integers(0, 256, (16, 3), np.uint8)
    idx = rng.integers(0, 16, (6, 4, 1), np.uint8)
    assert np.array_equal(G._png_rgb(_png(idx, ctype=3, palette=pal)), pal[idx[..., 0]])
    with pytest.raises(ValueError):
        G._png_rgb(b"\xff\xd8\xff\xe0")


def _write_gltf(d, binary=False):
    """Two meshes (indexed uint16 and uint32, one without normals and uvs),
    three materials (textured, emissive with strength, transmissive with
    ior), a camera node with T and R, mesh nodes with a matrix and with TRS,
    and a child node that the importer must skip."""
    rng = np.random.default_rng(5)
    quad_p = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
    quad_n = np.tile(np.array([0, 1, 0], np.float32), (4, 1))
    quad_uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    quad_i = np.array([0, 2, 1, 0, 3, 2], np.uint16)
    tet_p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32) * 0.6
    tet_i = np.array([0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3], np.uint32)
    parts = [quad_p.tobytes(), quad_n.tobytes(), quad_uv.tobytes(), quad_i.tobytes() + b"\0\0",
             tet_p.tobytes(), tet_i.tobytes()]
    offs = np.cumsum([0] + [len(p) for p in parts])
    blob = b"".join(parts)
    views = [dict(buffer=0, byteOffset=int(offs[k]), byteLength=len(parts[k])) for k in range(6)]
    acc = [dict(bufferView=0, componentType=5126, count=4, type="VEC3"),
           dict(bufferView=1, componentType=5126, count=4, type="VEC3"),
           dict(bufferView=2, componentType=5126, count=4, type="VEC2"),
           dict(bufferView=3, componentType=5123, count=6, type="SCALAR"),
           dict(bufferView=4, componentType=5126, count=4, type="VEC3"),
           dict(bufferView=5, componentType=5125, count=12, type="SCALAR")]
    tex = rng.integers(0, 256, (8, 8, 3), np.uint8)
    png = _png(tex)
    with open(os.path.join(d, "albedo.png"), "wb") as f:
        f.write(png)
    emis = rng.integers(0, 256, (4, 4, 4), np.uint8)
    doc = dict(
        asset=dict(version="2.0"),
        scenes=[dict(nodes=[0, 1, 2])],
        nodes=[dict(camera=0, translation=[0.0, 1.5, 4.0], rotation=[-0.1, 0.0, 0.0, 0.995]),
               dict(mesh=0, matrix=[2, 0, 0, 0, 0, 1, 0, 0, 0, 0, 2, 0, 0, -0.5, 0, 1]),
               dict(mesh=1, translation=[0.3, 0.2, 0.1], rotation=[0, 0.3826834, 0, 0.9238795],
                    scale=[1.5, 1.5, 1.5], children=[3]),
               dict(mesh=1, translation=[5.0, 5.0, 5.0])],
        cameras=[dict(type="perspective", perspective=dict(yfov=0.8, znear=0.1, aspectRatio=1.5))],
        meshes=[dict(primitives=[dict(attributes=dict(POSITION=0, NORMAL=1, TEXCOORD_0=2), indices=3, material=0)]),
                dict(primitives=[dict(attributes=dict(POSITION=4), indices=5, material=1),
                                 dict(attributes=dict(POSITION=4), indices=5, material=2)])],
        materials=[dict(pbrMetallicRoughness=dict(baseColorFactor=[0.9, 0.8, 0.7, 1.0], metallicFactor=0.0,
                                                  roughnessFactor=0.6, baseColorTexture=dict(index=0))),
                   dict(emissiveFactor=[1.0, 0.5, 0.25], emissiveTexture=dict(index=1),
                        extensions=dict(KHR_materials_emissive_strength=dict(emissiveStrength=12.0)),
                        pbrMetallicRoughness=dict(metallicFactor=0.0)),
                   dict(pbrMetallicRoughness=dict(baseColorFactor=[0.95, 0.95, 1.0, 1.0], metallicFactor=0.0,
                                                  roughnessFactor=0.1),
                        extensions=dict(KHR_materials_transmission=dict(transmissionFactor=1.0),
                                        KHR_materials_ior=dict(ior=1.5)))],
        textures=[dict(source=0), dict(source=1)],
        images=[dict(uri="albedo.png"),
                dict(uri="data:image/png;base64," + base64.b64encode(_png(emis)).decode())],
        bufferViews=views, accessors=acc,
        buffers=[dict(byteLength=len(blob))])
    if binary:
        # the image of the first texture and the geometry in the BIN chunk
        doc["bufferViews"].append(dict(buffer=0, byteOffset=len(blob), byteLength=len(png)))
        doc["images"][0] = dict(bufferView=6, mimeType="image/png")
        blob = blob + png
        blob += b"\0" * (-len(blob) % 4)
        doc["buffers"][0]["byteLength"] = len(blob)
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        out = os.path.join(d, "scene.glb")
        with open(out, "wb") as f:
            f.write(struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(blob)))
            f.write(struct.pack("<II", len(js), 0x4E4F534A) + js)
            f.write(struct.pack("<II", len(blob), 0x004E4942) + blob)
        return out, tex, emis
    with open(os.path.join(d, "scene.bin"), "wb") as f:
        f.write(blob)
    doc["buffers"][0]["uri"] = "scene.bin"
    out = os.path.join(d, "scene.gltf")
    with open(out, "w") as f:
        json.dump(doc, f)
    return out, tex, emis


def test_gltf_scene_mapping(tmp_path):
    path, tex, emis = _write_gltf(str(tmp_path))
    sc = G.load_gltf(path, 64, 48)
    assert len(sc.meshes) == 2 and len(sc.instances) == 2       # the child node is skipped
    q = sc.meshes[0]
    assert q.ntris == 2 and np.array_equal(q.material, [0, 0])
    np.testing.assert_array_equal(q.positions[0], [[-1, 0, -1], [1, 0, 1], [1, 0, -1]])
    np.testing.assert_array_equal(q.uvs[1], [[0, 0], [0, 1], [1, 1]])
    t = sc.meshes[1]
    assert t.ntris == 8 and np.array_equal(t.material, [1] * 4 + [2] * 4)
    assert np.allclose(np.linalg.norm(t.normals, axis=2), 1.0)  # flat normals where the file has none
    np.testing.assert_array_equal(sc.instances[0].model, np.diag([2, 1, 2, 1]) + np.array(
        [[0, 0, 0, 0], [0, 0, 0, -0.5], [0, 0, 0, 0], [0, 0, 0, 0]]))
    c, s_ = math.cos(math.pi / 4), math.sin(math.pi / 4)
    rot = np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]])
    np.testing.assert_allclose(sc.instances[1].model[:3, :3], rot * 1.5, atol=1e-6)
    np.testing.assert_allclose(sc.instances[1].model[:3, 3], [0.3, 0.2, 0.1], atol=1e-7)
    m = sc.materials
    assert len(m) == 4                                         # + the default material
    assert m[0]["albedo_tex"] == 0 and np.allclose(m[0]["albedo"], [0.9, 0.8, 0.7]) and m[0]["roughness"] == \
        np.float32(0.6)
    assert m[1]["emission_tex"] == 1 and m[1]["emission_scale"] == 12.0 and np.allclose(m[1]["emission"],
                                                                                      [1, 0.5, 0.25])
    assert m[2]["transmission"] == 1.0 and m[2]["ior"] == np.float32(1.5) and m[2]["emission_scale"] == 0.0
    assert m[0]["ior"] == np.float32(1.45) and m[3]["metallic"] == 1.0
    assert np.array_equal(sc.textures[0], tex) and np.array_equal(sc.textures[1], emis[..., :3])
    # camera: inverse view = T * R with its third column negated
    qv = np.array([-0.1, 0.0, 0.0, 0.995]) / np.linalg.norm([-0.1, 0.0, 0.0, 0.995])
    model = S.translate(0.0, 1.5, 4.0) @ G._quat(qv)
    iv = model.copy()
    iv[:, 2] *= -1
    np.testing.assert_allclose(sc.camera.inv_view, iv, atol=1e-6)
    np.testing.assert_allclose(np.linalg.inv(sc.camera.inv_proj), S.perspective_fov_lh(0.8, 100, 100, 1, 100),
                               rtol=1e-5, atol=1e-6)


def test_glb_matches_gltf(tmp_path):
    a = G.load_gltf(_write_gltf(str(tmp_path))[0], 32, 32)
    b = G.load_gltf(_write_gltf(str(tmp_path), binary=True)[0], 32, 32)
    for ma, mb in zip(a.meshes, b.meshes):
        for f in ("positions", "normals", "uvs", "material"):
            assert np.array_equal(getattr(ma, f), getattr(mb, f))
    assert a.materials.tobytes() == b.materials.tobytes()
    assert all(np.array_equal(x, y) for x, y in zip(a.textures, b.textures))
    assert np.array_equal(a.camera.inv_view, b.camera.inv_view)


@pytest.mark.gpu
def test_gltf_scene_renders_like_oracle(tmp_path):
    from oracle import oracle as O
    from tests.test_gpu_parity import make_renderer, render_samples
    sc = G.load_gltf(_write_gltf(str(tmp_path), binary=True)[0], 64, 48, max_depth=4)
    sc.env["sun_theta"] = 0.6
    r = make_renderer(sc)
    try:
        rad, hit, alb = render_samples(r, sc, 2)
    finally:
        r.shutdown()
    ref = O.Scene(sc).render_samples(0, 2)
    assert (ref["first_hit"][..., 0] >= 0).mean() > 0.2
    err = np.abs(rad - ref["radiance"]).max(-1) / np.maximum(np.abs(ref["radiance"]).max(-1), 1e-3)
    assert (err <= 1e-4).mean() >= 0.99
    # visible-surface albedo: textured surfaces decode sRGB texels with the
    # path kernels' fast powf, so within 1e-5 rather than bit for bit
    m = hit[..., 0] >= 0
    np.testing.assert_allclose(alb[m], ref["albedo"][m], rtol=1e-5, atol=1e-7)
