"""Scene loading (kgk_load_obj, kgk_load_image) against the reference's own
loader: load_object / load_Textures (FileIO/IO_load_WavefrontObj.cuh:10-127,
tinyobjloader) and stbi_loadf (FileIO/IO_load_images.cuh:9-19, stb_image),
compiled for the host.  The committed fixture tests/golden/loader_ref.npz
holds the reference's outputs for the seeded files that
tests/golden/scene_files.py writes; when oracle/_ref is built the reference
is also run live.  Bar: bit-exact (triangles, materials, every float pixel).
Host-only: no GPU needed.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden
from kagayaki_gb300 import KgkError, load_image, load_obj, scenes

sys.path.insert(0, GOLDEN)
import scene_files  # noqa: E402


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return (a.shape == b.shape and a.dtype.itemsize == b.dtype.itemsize and
            np.array_equal(a.view(np.uint8), b.view(np.uint8)))


def test_images_match_stb_loadf(tmp_path):
    g = golden("loader_ref.npz")
    names = scene_files.write_images(str(tmp_path))
    assert len(names) >= 30
    for name in names:
        ours = load_image(tmp_path / name)
        assert same_bits(ours, g["img_" + name]), name


def test_obj_scene_matches_reference_loader(tmp_path):
    g = golden("loader_ref.npz")
    path = scene_files.write_obj_scene(str(tmp_path))
    tris, mats, texs, env = load_obj(path)
    assert env is None
    assert same_bits(scenes.canonical(tris), scenes.canonical(g["obj_tris"]))  # padding bytes zeroed
    assert same_bits(mats, g["obj_mats"])
    assert len(texs) == int(g["obj_ntex"])
    for i, t in enumerate(texs):
        assert same_bits(t, g[f"obj_tex{i}"]), i
    # what the scene exercises
    assert set(np.unique(tris["shape_id"])) == {0, 1, 2, 4}  # shape 3 has only lines, but it counts
    assert set(np.unique(tris["material_id"])) >= {0, 1, 2, 3, 4, 5}
    assert tris["is_SmoothNormal"].any() and not tris["is_SmoothNormal"].all()


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libkgkref.so")), reason="reference build not present")
def test_live_against_reference_build(tmp_path):
    from oracle import orc
    names = scene_files.write_images(str(tmp_path))
    for name in names:
        assert same_bits(load_image(tmp_path / name), orc.ref_load_image(str(tmp_path / name))), name
    scene_files.write_obj_scene(str(tmp_path))
    rt, rm, rx = orc.ref_load_obj(str(tmp_path))
    tris, mats, texs, _ = load_obj(tmp_path / "OBJ.obj")
    assert same_bits(scenes.canonical(tris), scenes.canonical(rt))
    assert same_bits(mats, rm)
    for a, b in zip(texs, rx):
        assert same_bits(a, b)


def test_environment_loaded_without_offset(tmp_path):
    g = golden("loader_ref.npz")
    scene_files.write_images(str(tmp_path))
    path = scene_files.write_obj_scene(str(tmp_path))
    _, _, _, env = load_obj(path, tmp_path / "rle.hdr")
    assert same_bits(env, g["img_rle.hdr"])


def test_missing_normals_and_texcoords_are_tolerated(tmp_path):
    (tmp_path / "a.obj").write_text("v 0 0 0\nv 2 0 0\nv 0 3 0\nv 0 0 1\nf 1 2 3\nf 1 2/1 4\nvt 0.5 0.5\n")
    tris, mats, texs, _ = load_obj(tmp_path / "a.obj")
    assert len(tris) == 2 and len(mats) == 1 and not texs
    np.testing.assert_array_equal(tris["verts"][0, 3:6, :3], [[0, 0, 1]] * 3)  # face normal
    np.testing.assert_array_equal(tris["verts"][1, 3:6, :3], [[0, -1, 0]] * 3)
    assert np.all(tris["verts"][0, 6:9] == 0)  # no texcoords
    # a positive index may name a vt defined later in the file (resolved at the end)
    np.testing.assert_array_equal(tris["verts"][1, 6:9, :3], [[0, 0, 0], [0.5, 0.5, 0], [0, 0, 0]])


def test_errors(tmp_path):
    with pytest.raises(KgkError, match="cannot open"):
        load_obj(tmp_path / "missing.obj")
    (tmp_path / "bad.obj").write_text("v 0 0 0\nf 0 1 2\n")
    with pytest.raises(KgkError, match="bad face index"):
        load_obj(tmp_path / "bad.obj")
    (tmp_path / "oob.obj").write_text("v 0 0 0\nv 1 0 0\nf 1 2 7\n")
    with pytest.raises(KgkError, match="out of range"):
        load_obj(tmp_path / "oob.obj")
    (tmp_path / "x.jpg").write_bytes(b"\xff\xd8\xff\xe0" + bytes(64))
    with pytest.raises(KgkError, match="JPEG"):
        load_image(tmp_path / "x.jpg")


def png_header(w, h, ctype):
    """A PNG signature, an IHDR chunk for w x h at 8 bits of colour type
    `ctype`, and an empty IEND (no image data)."""
    import struct
    import zlib

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IEND", b""))


def test_image_format_errors(tmp_path):
    """The cases stb_image rejects are errors here too (no partial image)."""
    rng = np.random.default_rng(3)
    rgb = rng.integers(0, 256, (4, 5, 3), np.uint8)
    bmp = bytearray(scene_files.bmp_bytes(rgb, 24))
    bmp[30:34] = (1).to_bytes(4, "little")  # BI_RLE8
    cases = [("rle.bmp", bytes(bmp), "RLE"),
             ("gap.bmp", bytes(bmp[:10]) + (60).to_bytes(4, "little") + bytes(bmp[14:30]) + bytes(4) +
              bytes(bmp[34:54]) + bytes(6) + bytes(bmp[54:]), "offset"),
             ("cmyk.psd", scene_files.psd_bytes(rng.integers(0, 256, (4, 3, 3), np.uint8))[:24] +
              (4).to_bytes(2, "big") + scene_files.psd_bytes(rng.integers(0, 256, (4, 3, 3), np.uint8))[26:],
              "RGB"),
             ("noclear.gif", b"GIF89a\x02\x00\x02\x00\x80\x00\x00" + bytes(6) +
              b"\x2c\x00\x00\x00\x00\x02\x00\x02\x00\x00\x02\x02\x01\x00\x00\x3b", "clear code"),
             ("empty.gif", b"GIF89a\x02\x00\x02\x00\x00\x00\x00\x3b", "no image"),
             ("shortpal.tga", scene_files.tga_bytes(rng.integers(0, 4, (3, 3), np.uint8), 1, 8,
                                                    palette=rng.integers(0, 256, (4, 3), np.uint8),
                                                    pal_bits=24)[:24], "palette"),
             ("noise.bin", bytes(rng.integers(0, 256, 64, np.uint8)) + b"", "unknown image format"),
             # stb's size rule: width * height * channels must fit in an int
             ("huge.bmp", bytes(bmp[:18]) + (30000).to_bytes(4, "little") + (30000).to_bytes(4, "little") +
              bytes(bmp[26:30]) + bytes(4) + bytes(bmp[34:]), "too large"),
             ("huge.gif", b"GIF89a\xff\xff\xff\xff\x00\x00\x00\x3b", "too large"),
             # a few bytes claiming 40000 x 40000 RGBA: rejected before any allocation
             ("huge.png", png_header(40000, 40000, 6), "too large"),
             ("huge.hdr", b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 30000 +X 30000\n" + bytes(16), "too large")]
    for name, data, msg in cases:
        (tmp_path / name).write_bytes(data)
        with pytest.raises(KgkError, match=msg):
            load_image(tmp_path / name)


def test_parallel_parse_is_independent_of_threads(tmp_path):
    """The chunked parallel parse (relative indices, groups, materials and
    smoothing groups crossing chunk boundaries, mixed line ends) gives the
    sequential parse's result bit for bit."""
    scene_files.write_obj_scene(str(tmp_path))
    path = scene_files.write_big_obj(str(tmp_path), n_blocks=1500)
    assert os.path.getsize(path) > 3 << 20  # several 256 KB chunks at every thread count below
    t1, m1, x1, _ = load_obj(path, threads=1)  # one chunk: the sequential reader
    assert len(t1) > 50000 and len(np.unique(t1["shape_id"])) > 20
    for th in (2, 3, 7):
        t, m, x, _ = load_obj(path, threads=th)
        assert same_bits(scenes.canonical(t), scenes.canonical(t1)), th
        assert same_bits(m, m1)
        assert len(x) == len(x1) and all(same_bits(a, b) for a, b in zip(x, x1))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libkgkref.so")), reason="reference build not present")
def test_large_file_against_reference_build(tmp_path):
    from oracle import orc
    scene_files.write_obj_scene(str(tmp_path))
    path = scene_files.write_big_obj(str(tmp_path), n_blocks=600, seed=9, full_indices=True)
    os.replace(path, tmp_path / "OBJ.obj")  # the reference reads OBJ.obj from its directory
    rt, rm, _ = orc.ref_load_obj(str(tmp_path))
    tris, mats, _, _ = load_obj(tmp_path / "OBJ.obj", threads=4)
    assert same_bits(scenes.canonical(tris), scenes.canonical(rt))
    assert same_bits(mats, rm)


def test_pbr_materials_map_to_disney(tmp_path):
    from kagayaki_gb300 import MATERIALS_PBR, structs
    path = scene_files.write_obj_scene(str(tmp_path))
    with open(tmp_path / "scene.mtl", "a") as f:
        f.write("\nnewmtl coat\nKd 0.2 0.4 0.8\nPr 0.3\nPc 1.5\nPcr 0.25\nPs 0.5\naniso 0.7\n")
    with open(path, "a") as f:
        f.write("usemtl coat\nf 1 2 3\n")
    _, ref_m, _, _ = load_obj(path)
    tris, m, _, _ = load_obj(path, materials=MATERIALS_PBR)
    names = ["red", "tex_rgb", "emissive", "tex_ga", "tex_pal", "tex_jpg", "coat"]
    assert len(m) == len(ref_m) == len(names) + 1
    for i, name in enumerate(names, start=1):
        if name not in ("red", "coat"):  # no PBR key: converted as the reference does
            assert same_bits(m[i], ref_m[i]), name
    red, coat = m[1], m[7]
    assert red["MATERIAL_TYPE_ID"] == structs.DISNEY and coat["MATERIAL_TYPE_ID"] == structs.DISNEY
    np.testing.assert_allclose(red["diffuse"][:3], [0.63, 0.065, 0.05], rtol=1e-6)
    assert red["roughness"] == np.float32(0.5) and red["metallic"] == np.float32(0.25)
    f0 = ((1.33 - 1) / (1.33 + 1)) ** 2
    np.testing.assert_allclose(red["specular"], f0 / 0.08, rtol=1e-5)
    assert red["IOR"] == np.float32(1.33)
    assert coat["clearcoat"] == 1.0 and coat["cloearcoatGloss"] == np.float32(0.75)  # Pc clamped to 1
    assert coat["sheen"] == np.float32(0.5) and coat["anisotropic"] == np.float32(0.7)
    assert coat["specular"] == np.float32(0.5) and coat["IOR"] == np.float32(1.45)
    assert tris["material_id"][-1] == 7
    with pytest.raises(KgkError, match="material_model"):
        load_obj(path, materials=7)


def _normalize_ref(a):
    """Vec normalize (struct_Vec.cuh:40-46) in float32: a zero vector becomes (10000, 0, 0)."""
    a = a.astype(np.float32)
    x, y, z = a[..., 0], a[..., 1], a[..., 2]
    ln = np.sqrt(x * x + y * y + z * z)
    safe = np.where(ln == 0, np.float32(1), ln)
    out = a / safe[..., None]
    out[ln == 0] = np.array([10000, 0, 0], np.float32)
    return out


def test_vendored_models_parse_like_tinyobjloader():
    """Every test model vendored with tinyobjloader, parsed by the reference's
    own tinyobjloader build and by kgk_load_obj: the same accept / reject
    decision, and for accepted files the same triangles bit for bit -
    positions, normals (the file's when all three corners have one, else the
    face normal), texcoords, material ids (+1 for the reserved material),
    smooth flags and shape ids.  Models whose MTL names a texture image that
    is not among the models are skipped (the reference loads its textures
    too), as are files with no triangles (the library rejects those)."""
    from oracle import orc
    models = orc.ref_models_dir()
    if models is None:
        pytest.skip("reference build or checkout not present")
    compared = skipped_tex = 0
    for name in sorted(os.listdir(models)):
        if not name.endswith(".obj"):
            continue
        path = os.path.join(models, name)
        ref = orc.ref_tinyobj(path)
        try:
            tris, mats, _, _ = load_obj(path)
        except KgkError as e:
            if "cannot open image" in str(e):
                skipped_tex += 1
                continue
            assert ref is None or len(ref["face"]) == 0, (name, str(e))
            continue
        assert ref is not None and len(ref["face"]) == len(tris), name
        c = ref["corners"]
        P = ref["v"][c[:, :, 0]]
        assert same_bits(tris["verts"][:, 0:3, :3], P), name
        nn, nt = len(ref["vn"]), len(ref["vt"])
        ok_n = ((c[:, :, 2] >= 0) & (c[:, :, 2] < nn)).all(1)
        raw_n = ref["vn"][np.clip(c[:, :, 2], 0, max(nn - 1, 0))] if nn else np.zeros_like(P)
        e1, e2 = P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]
        face = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                         e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1)
        exp_n = np.where(ok_n[:, None, None], _normalize_ref(raw_n), _normalize_ref(face)[:, None, :])
        assert same_bits(tris["verts"][:, 3:6, :3], exp_n), name
        ok_t = (c[:, :, 1] >= 0) & (c[:, :, 1] < nt)
        raw_t = ref["vt"][np.clip(c[:, :, 1], 0, max(nt - 1, 0))] if nt else np.zeros(c.shape[:2] + (2,), np.float32)
        exp_t = np.zeros(c.shape[:2] + (3,), np.float32)
        exp_t[..., :2] = np.where(ok_t[..., None], raw_t, 0)
        assert same_bits(tris["verts"][:, 6:9, :3], exp_t), name
        assert np.array_equal(tris["material_id"], ref["face"][:, 0] + 1), name
        assert np.array_equal(tris["is_SmoothNormal"], ref["face"][:, 1] != 0), name
        assert np.array_equal(tris["shape_id"], ref["face"][:, 2]), name
        assert len(mats) == ref["n_materials"] + 1, name
        compared += 1
    assert compared >= 25 and skipped_tex <= 10, (compared, skipped_tex)
