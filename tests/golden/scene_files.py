"""Seeded scene and image files for the loader tests (TEST INFRASTRUCTURE).

Writes, into a directory, the inputs that tests/test_loader.py reads with the
library and tests/golden/make_golden.py reads with the reference's own loader
(load_object / stbi_loadf compiled for the host):

  images: PNG in every colour type and bit depth (random row filters, zlib
          compression, Adam7 interlacing, tRNS), binary PNM, Radiance .hdr
          (flat and run-length scanlines)
  OBJ.obj + scene.mtl + textures: triangles, quads, convex and concave
          polygons, negative indices, groups / objects, smoothing groups,
          usemtl switches (including an unknown material), numbers in several
          notations, textured and untextured materials.
"""
import os
import struct
import zlib

import numpy as np

# ---------------------------------------------------------------------------
# PNG
# ---------------------------------------------------------------------------
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xffffffff)


def _pack_row(samples, depth):
    """samples: 1-D ints of one row (all channels) -> bytes."""
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in samples)
    if depth == 8:
        return bytes(int(v) for v in samples)
    per = 8 // depth
    out = bytearray((len(samples) + per - 1) // per)
    for i, v in enumerate(samples):
        out[i // per] |= (int(v) & ((1 << depth) - 1)) << (8 - depth * (i % per + 1))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_rows(rows, bpp, rng):
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for r in rows:
        ft = int(rng.integers(0, 5))
        f = bytearray(len(r))
        for i in range(len(r)):
            a = r[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            f[i] = (r[i] - pred) & 255
        out.append(ft)
        out += f
        prev = r
    return bytes(out)


def png_bytes(img, ctype, depth, interlace=False, palette=None, trns=None, seed=0, level=6):
    """img: (h, w, channels) integer samples as stored (palette indices for
    colour type 3)."""
    rng = np.random.default_rng(seed)
    h, w, c = img.shape
    bpp = max(1, c * depth // 8)
    raw = b""
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for xo, yo, xs, ys in passes:
        sub = img[yo::ys, xo::xs]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = [_pack_row(sub[j].reshape(-1), depth) for j in range(sub.shape[0])]
        raw += _filter_rows(rows, bpp, rng)
    comp = zlib.compress(raw, level)
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        out += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += _chunk(b"tRNS", bytes(trns))
    half = len(comp) // 2
    out += _chunk(b"IDAT", comp[:half]) + _chunk(b"IDAT", comp[half:])  # two IDAT chunks
    out += _chunk(b"tEXt", b"Comment\x00seeded test image")
    return out + _chunk(b"IEND", b"")


def png_cases():
    """(name, bytes) for every colour type / depth / interlace / tRNS combination."""
    rng = np.random.default_rng(11)
    cases = []
    k = 0
    for ctype, depths in ((0, (1, 2, 4, 8, 16)), (2, (8, 16)), (3, (1, 2, 4, 8)), (4, (8, 16)), (6, (8, 16))):
        ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
        for depth in depths:
            for interlace in (False, True):
                w, h = int(rng.integers(5, 19)), int(rng.integers(3, 14))
                if ctype == 3:
                    npal = int(rng.integers(2, (1 << depth) + 1)) if depth < 8 else 200
                    img = rng.integers(0, npal, (h, w, 1))
                    pal = rng.integers(0, 256, (npal, 3))
                    trns = bytes(rng.integers(0, 256, max(1, npal // 2)).tolist()) if k % 2 == 0 else None
                    cases.append((f"pal_d{depth}_i{int(interlace)}.png",
                                  png_bytes(img, 3, depth, interlace, palette=pal, trns=trns, seed=k)))
                else:
                    img = rng.integers(0, 1 << depth, (h, w, ch))
                    trns = None
                    if ctype in (0, 2) and k % 2 == 1:
                        key = img[0, 0]
                        trns = b"".join(struct.pack(">H", int(v)) for v in key)
                    cases.append((f"c{ctype}_d{depth}_i{int(interlace)}.png",
                                  png_bytes(img, ctype, depth, interlace, trns=trns, seed=k, level=k % 10)))
                k += 1
    # a stored (uncompressed) stream and a fixed-Huffman stream
    img = rng.integers(0, 256, (6, 9, 3))
    cases.append(("c2_stored.png", png_bytes(img, 2, 8, seed=99, level=0)))
    return cases


# ---------------------------------------------------------------------------
# Radiance .hdr and PNM
# ---------------------------------------------------------------------------
def to_rgbe(rgb):
    rgb = np.asarray(rgb, np.float64)
    m = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    nz = m > 1e-32
    mant, ex = np.frexp(m[nz])
    scale = mant * 256.0 / m[nz]
    out[nz, :3] = np.clip(np.floor(rgb[nz] * scale[:, None]), 0, 255).astype(np.uint8)
    out[nz, 3] = (ex + 128).astype(np.uint8)
    return out


def _rle_component(vals):
    out = bytearray()
    i, n = 0, len(vals)
    while i < n:
        run = 1
        while i + run < n and run < 127 and vals[i + run] == vals[i]:
            run += 1
        if run >= 3:
            out += bytes([128 + run, vals[i]])
            i += run
        else:
            j = i
            while j < n and j - i < 128 and not (j + 2 < n and vals[j] == vals[j + 1] == vals[j + 2]):
                j += 1
            out += bytes([j - i]) + bytes(vals[i:j])
            i = j
    return bytes(out)


def hdr_bytes(rgb, rle=True, magic="#?RADIANCE"):
    h, w, _ = rgb.shape
    e = to_rgbe(rgb)
    out = (magic + "\n# seeded test image\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n" + f"-Y {h} +X {w}\n").encode()
    for j in range(h):
        if rle:
            out += bytes([2, 2, w >> 8, w & 255])
            for k in range(4):
                out += _rle_component(list(e[j, :, k]))
        else:
            out += e[j].tobytes()
    return out


def hdr_cases():
    rng = np.random.default_rng(12)
    cases = []
    base = rng.uniform(0, 4, (9, 23, 3))
    base[:, 5:15] = base[:, 5:6]  # runs for the RLE coder
    base[3, 2] = 0.0
    base[4, 7] = (1e4, 2e3, 10.0)
    cases.append(("rle.hdr", hdr_bytes(base, True)))
    cases.append(("flat_wide.hdr", hdr_bytes(base, False, "#?RGBE")))  # width >= 8 without RLE headers
    cases.append(("flat_narrow.hdr", hdr_bytes(rng.uniform(0, 2, (5, 6, 3)), False)))
    return cases


def pnm_cases():
    rng = np.random.default_rng(13)
    g = rng.integers(0, 256, (7, 10), np.uint8)
    c = rng.integers(0, 256, (5, 8, 3), np.uint8)
    c16 = rng.integers(0, 65536, (4, 6, 3)).astype(">u2")
    return [("gray.pgm", b"P5\n# comment\n10 7\n255\n" + g.tobytes()),
            ("rgb.ppm", b"P6 8 5 255\n" + c.tobytes()),
            ("rgb16.ppm", b"P6\n6 4\n65535\n" + c16.tobytes())]


def image_cases():
    return png_cases() + hdr_cases() + pnm_cases()


# ---------------------------------------------------------------------------
# OBJ + MTL + textures
# ---------------------------------------------------------------------------
OBJ_TEXT = """# seeded loader test scene
mtllib scene.mtl
o box
v 0 0 0
v 1.0 0 0
v 1 1.5e0 0
v 0 1 0
v -.25 0.5 1.25
v 0.5 +2 3.14159265358979
v 1e-3 -0.125 7.0000001
v 123.456789 0.0000000123 -4.5E+1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vt .5 .25
vn 0 0 1
vn 0 0 -2
vn 1 1 1
vn 0.3 -0.4 0.5
usemtl red
s 1
f 1/1/1 2/2/1 3/3/1
f 1/1/2 3/3/2 4/4/2 5/5/2
s off
usemtl tex_rgb
f -8/-5/-4 -7/-4/-3 -6/-3/-2 -5/-2/-1
g second group
usemtl no_such_material
f 5/5/3 6/1/3 7/2/3 8/3/3 1/4/3
s 2
usemtl emissive
f 2/1/4 3/2/4 4/3/4
o star
v 0 0 5
v 2 0.4 5
v 4 0 5
v 3.6 2 5
v 4 4 5
v 2 3.6 5
v 0 4 5
v 0.4 2 5
vn 0 0 1
usemtl tex_ga
f 9/1/5 10/2/5 11/3/5 12/4/5 13/5/5 14/1/5 15/2/5 16/3/5
usemtl tex_pal
f 9/1/5 11/3/5 13/5/5
l 1 2 3
o lines_only
l 9 10
o last
usemtl red
f 16/4/5 15/3/5 14/2/5 13/1/5 12/5/5 11/4/5
"""

MTL_TEXT = """# materials
newmtl red
Kd 0.63 0.065 0.05
Ks 0.1 0.2 0.3
Pr 0.5
Pm 0.25
Ni 1.33
illum 2

newmtl tex_rgb
map_Kd tex_rgb.png
Ks 0.5 0.5 0.5

newmtl emissive
Kd 0 0.5 0.5
Ke 17 12 4

newmtl tex_ga
Kd 1 1 1
map_Kd some/dir/tex_ga.png

newmtl tex_pal
Kd 0.2 0.3 0.4
map_Kd -blendu off -s 1 1 1 tex_pal.png
"""


def write_obj_scene(d):
    rng = np.random.default_rng(14)
    with open(os.path.join(d, "OBJ.obj"), "w") as f:
        f.write(OBJ_TEXT)
    with open(os.path.join(d, "scene.mtl"), "w") as f:
        f.write(MTL_TEXT)
    with open(os.path.join(d, "tex_rgb.png"), "wb") as f:
        f.write(png_bytes(rng.integers(0, 256, (16, 12, 3)), 2, 8, seed=1))
    with open(os.path.join(d, "tex_ga.png"), "wb") as f:
        f.write(png_bytes(rng.integers(0, 65536, (9, 7, 2)), 4, 16, interlace=True, seed=2))
    with open(os.path.join(d, "tex_pal.png"), "wb") as f:
        f.write(png_bytes(rng.integers(0, 12, (5, 11, 1)), 3, 4, palette=rng.integers(0, 256, (12, 3)),
                          trns=bytes([0, 128, 255]), seed=3))
    return os.path.join(d, "OBJ.obj")


def write_big_obj(d, n_blocks=2000, seed=5, full_indices=False):
    """A large seeded OBJ for the parallel parser: blocks of vertices and
    faces (triangles to hexagons, absolute and relative indices, with and
    without vt / vn) separated by group, object, material, smoothing, line and
    point records, comments and blank lines, with \\n, \\r\\n and \\r line ends
    mixed.  full_indices: every corner has v/vt/vn (the reference's loader
    needs both).  Uses scene.mtl of write_obj_scene."""
    rng = np.random.default_rng(seed)
    out = ["mtllib scene.mtl\n"]
    nv = nvt = nvn = 0
    ends = ["\n", "\r\n", "\r"]
    mats = ["red", "tex_rgb", "emissive", "tex_ga", "no_such_material"]
    for b in range(n_blocks):
        le = ends[int(rng.integers(0, 3))]
        k = int(rng.integers(8, 40))
        pts = rng.normal(0, 10, (k, 3)) + rng.normal(0, 100, 3)
        out.append("".join(f"v {x:.6f} {y:.6f} {z:.6f}{le}" for x, y, z in pts))
        out.append("".join(f"vt {u:.5f} {v:.5f}{le}" for u, v in rng.random((k // 2, 2))))
        out.append("".join(f"vn {x:.4f} {y:.4f} {z:.4f}{le}" for x, y, z in rng.normal(0, 1, (k // 3, 3))))
        nv += k
        nvt += k // 2
        nvn += k // 3
        for f in range(int(rng.integers(10, 60))):
            r = rng.random()
            if r < 0.03:
                out.append(rng.choice([f"g grp{b}_{f}", f"o obj{b}_{f}", "g", "# comment", "", "   "]) + le)
            elif r < 0.07:
                out.append(f"usemtl {mats[int(rng.integers(0, len(mats)))]}{le}")
            elif r < 0.10:
                out.append(rng.choice(["s 1", "s off", "s 0", "s 3"]) + le)
            elif r < 0.11:
                out.append(f"l {int(rng.integers(1, nv + 1))} {int(rng.integers(1, nv + 1))}{le}")
            elif r < 0.115:
                out.append(f"p {-int(rng.integers(1, k + 1))}{le}")
            n = int(rng.choice([3, 3, 3, 4, 4, 5, 6]))
            corners = []
            style = int(rng.integers(0, 4)) if not full_indices else 3
            for c in range(n):
                rel = rng.random() < 0.3
                iv = int(rng.integers(1, k + 1))  # within this block, so convex-ish faces stay local
                v = -iv if rel else nv - k + iv
                t = -int(rng.integers(1, k // 2 + 1)) if rel else int(rng.integers(1, nvt + 1))
                m = -int(rng.integers(1, k // 3 + 1)) if rel else int(rng.integers(1, nvn + 1))
                corners.append([f"{v}", f"{v}/{t}", f"{v}//{m}", f"{v}/{t}/{m}"][style])
            out.append("f " + " ".join(corners) + le)
    path = os.path.join(d, "big.obj")
    with open(path, "w", newline="") as f:
        f.write("".join(out))
    return path


def write_images(d):
    names = []
    for name, data in image_cases():
        with open(os.path.join(d, name), "wb") as f:
            f.write(data)
        names.append(name)
    return names
