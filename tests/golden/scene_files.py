"""Seeded scene and image files for the loader tests (TEST INFRASTRUCTURE).

Writes, into a directory, the inputs that tests/test_loader.py reads with the
library and tests/golden/make_golden.py reads with the reference's own loader
(load_object / stbi_loadf compiled for the host):

  images: PNG in every colour type and bit depth (random row filters, zlib
          compression, Adam7 interlacing, tRNS), binary PNM, Radiance .hdr
          (flat and run-length scanlines), JPEG, BMP (every header size and
          bit depth, bit fields), TGA (raw / run-length, grey, paletted,
          15/16-bit), GIF (LZW with table restarts, interlacing, local
          palettes, transparency, background fill), PSD (raw / RLE, 8 and 16
          bits) and Softimage PIC (raw, pure and mixed run-length packets)
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


# ---------------------------------------------------------------------------
# JPEG (a small encoder for the fixtures: any sampling factors, sequential
# interleaved or per-component scans, progressive spectral selection and
# successive approximation, restart intervals, Adobe / JFIF segments)
# ---------------------------------------------------------------------------
def _zigzag():
    order = []
    for s in range(15):
        rng_ = range(s + 1)
        for k in rng_:
            x = s - k if s % 2 else k
            y = s - x
            if x < 8 and y < 8:
                order.append(y * 8 + x)
    return np.array(order)


ZIGZAG = _zigzag()


def _dct_matrix():
    m = np.zeros((8, 8))
    for k in range(8):
        a = np.sqrt(1 / 8) if k == 0 else np.sqrt(2 / 8)
        for n in range(8):
            m[k, n] = a * np.cos((2 * n + 1) * k * np.pi / 16)
    return m


DCT8 = _dct_matrix()


def _huff_table(freq):
    """Code lengths (counts per length 1..16, symbols in order) for symbol
    frequencies by the JPEG standard's procedure (Annex K.2): a reserved
    dummy symbol keeps any code from being all ones, lengths above 16 are
    folded back."""
    freq = dict(freq)
    syms = sorted(freq)
    f = {k: v for k, v in freq.items() if v > 0}
    if not f:
        f = {0: 1}
    f[256] = 1  # reserved
    size = {k: 0 for k in f}
    others = {k: -1 for k in f}
    fr = dict(f)
    while True:
        live = [k for k in fr if fr[k] > 0]
        if len(live) < 2:
            break
        live.sort(key=lambda k: (fr[k], -k))
        c1, c2 = live[0], live[1]
        # c1: the least frequent (largest value on ties), c2: the next
        fr[c1] += fr[c2]
        fr[c2] = 0
        size[c1] += 1
        while others[c1] != -1:
            c1 = others[c1]
            size[c1] += 1
        others[c1] = c2
        size[c2] += 1
        while others[c2] != -1:
            c2 = others[c2]
            size[c2] += 1
    bits = [0] * 33
    for k, sz in size.items():
        bits[sz] += 1
    i = 32
    while i > 16:
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
        i -= 1
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # remove the reserved code
    vals = sorted((k for k in size if k != 256), key=lambda k: (size[k], k))
    counts = bits[1:17]
    # canonical codes
    codes = {}
    code = 0
    k = 0
    for ln in range(1, 17):
        for _ in range(counts[ln - 1]):
            codes[vals[k]] = (code, ln)
            code += 1
            k += 1
        code <<= 1
    return counts, vals, codes


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, code, length):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((code >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xff:
                    self.out.append(0)
                self.acc = 0
                self.n = 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _mag(v):
    a = abs(int(v))
    n = a.bit_length()
    bits = a if v >= 0 else (~a) & ((1 << n) - 1)
    return n, bits


def jpeg_bytes(planes, samp, qscale=1.0, scans=None, progressive=False, restart=0, adobe=None, jfif=True,
               ids=None, dqt16=False, pad_ff=False):
    """planes: component sample planes (uint8 arrays, component sizes of the
    image (W, H) for the sampling factors `samp` [(h, v), ...]).  scans:
    [(component indices, Ss, Se, Ah, Al)] (sequential: Ss=0, Se=63, A=0)."""
    nc = len(planes)
    hmax = max(h for h, _ in samp)
    vmax = max(v for _, v in samp)
    Hc = planes[0].shape[0] * vmax // samp[0][1] if False else None
    # image size from the first component (chosen with h = hmax, v = vmax by the callers)
    H, W = planes[0].shape
    mcux = -(-W // (8 * hmax))
    mcuy = -(-H // (8 * vmax))
    ids = ids or list(range(1, nc + 1))
    # quantisation: two procedural tables
    uu, vv = np.meshgrid(np.arange(8), np.arange(8))
    qt = [np.clip(np.round((2 + (uu + vv) * 2.5) * qscale), 1, 65535 if dqt16 else 255).astype(np.int64),
          np.clip(np.round((3 + (uu + vv) * 4.0) * qscale), 1, 65535 if dqt16 else 255).astype(np.int64)]
    tq = [0 if c == 0 else 1 for c in range(nc)]
    # coefficients per component: padded to whole MCUs with edge replication
    coefs = []
    for c in range(nc):
        h, v = samp[c]
        bw, bh = mcux * h, mcuy * v
        pl = planes[c].astype(np.float64)
        pad = np.pad(pl, ((0, bh * 8 - pl.shape[0]), (0, bw * 8 - pl.shape[1])), mode="edge")
        blocks = pad.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3) - 128.0
        d = np.einsum("ki,abij,lj->abkl", DCT8, blocks, DCT8)
        q = qt[tq[c]][None, None]
        coefs.append(np.round(d / q).astype(np.int64).reshape(bh, bw, 64))
    if scans is None:
        scans = [(list(range(nc)), 0, 63, 0, 0)]

    def blocks_of(comps):
        """(component, block row, block col) in scan order, MCU by MCU."""
        if len(comps) == 1:
            c = comps[0]
            h, v = samp[c]
            cw = -(-W * h // hmax)
            ch = -(-H * v // vmax)
            for by in range(-(-ch // 8)):
                for bx in range(-(-cw // 8)):
                    yield [(c, by, bx)]
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    unit = []
                    for c in comps:
                        h, v = samp[c]
                        for y in range(v):
                            for x in range(h):
                                unit.append((c, my * v + y, mx * h + x))
                    yield unit

    def pt_ac(val, al):  # point transform of an AC coefficient (magnitude shift)
        return -((-val) >> al) if val < 0 else val >> al

    def encode_scan(comps, ss, se, ah, al, tables=None):
        """Symbols of one scan: returns (dc freq, ac freq, writer) - with
        tables=None only counts symbols."""
        dcf, acf = {}, {}
        bw = _BitWriter()
        emit = tables is not None

        def sym(kind, s, extra=0, nbits=0):
            (dcf if kind == 0 else acf)[s] = (dcf if kind == 0 else acf).get(s, 0) + 1
            if emit:
                code, ln = tables[kind][s]
                bw.put(code, ln)
                if nbits:
                    bw.put(extra, nbits)

        state = {"eobrun": 0, "be": []}

        def flush_eob():
            r = state["eobrun"]
            if r:
                nb = r.bit_length() - 1
                sym(1, nb << 4, r - (1 << nb), nb)
                state["eobrun"] = 0
            if emit:
                for bit in state["be"]:
                    bw.put(bit, 1)
            state["be"] = []

        pred = {c: 0 for c in comps}
        units = list(blocks_of(comps))
        for ui, unit in enumerate(units):
            if restart and ui and ui % restart == 0:
                flush_eob()
                if emit:
                    bw.flush()
                    bw.out += bytes([0xff, 0xd0 + ((ui // restart - 1) % 8)])
                pred = {c: 0 for c in comps}
            for (c, by, bx) in unit:
                z = coefs[c][by, bx][ZIGZAG]
                if ss == 0:  # DC
                    if ah == 0:
                        dcv = int(z[0]) >> al
                        diff = dcv - pred[c]
                        pred[c] = dcv
                        n, bits = _mag(diff)
                        sym(0, n, bits, n)
                    else:
                        if emit:
                            bw.put((int(z[0]) >> al) & 1, 1)
                    if not progressive:  # sequential: the AC terms follow
                        r = 0
                        for k in range(1, 64):
                            v = int(z[k])
                            if v == 0:
                                r += 1
                                continue
                            while r > 15:
                                sym(1, 0xf0)
                                r -= 16
                            n, bits = _mag(v)
                            sym(1, (r << 4) | n, bits, n)
                            r = 0
                        if r:
                            sym(1, 0)
                    continue
                if ah == 0:  # AC first scan of the band
                    vals = [pt_ac(int(z[k]), al) for k in range(ss, se + 1)]
                    if not any(vals):
                        state["eobrun"] += 1
                        if state["eobrun"] == 0x7fff:
                            flush_eob()
                        continue
                    flush_eob()
                    r = 0
                    last = max(i for i, v in enumerate(vals) if v)
                    for i, v in enumerate(vals):
                        if i > last:
                            break
                        if v == 0:
                            r += 1
                            continue
                        while r > 15:
                            sym(1, 0xf0)
                            r -= 16
                        n, bits = _mag(v)
                        sym(1, (r << 4) | n, bits, n)
                        r = 0
                    if last < se - ss:
                        state["eobrun"] += 1
                        if state["eobrun"] == 0x7fff:
                            flush_eob()
                    continue
                # AC refinement scan (the standard's correction-bit scheme)
                absv = [abs(int(z[k])) >> al for k in range(ss, se + 1)]
                sign = [int(z[k]) >= 0 for k in range(ss, se + 1)]
                eob = max([i for i, v in enumerate(absv) if v == 1], default=-1)
                r = 0
                br = []
                for i, v in enumerate(absv):
                    if v == 0:
                        r += 1
                        continue
                    while r > 15 and i <= eob:
                        flush_eob()
                        sym(1, 0xf0)
                        r -= 16
                        if emit:
                            for bit in br:
                                bw.put(bit, 1)
                        br = []
                    if v > 1:
                        br.append(v & 1)
                        continue
                    flush_eob()
                    sym(1, (r << 4) | 1, 1 if sign[i] else 0, 1)
                    if emit:
                        for bit in br:
                            bw.put(bit, 1)
                    br = []
                    r = 0
                if r > 0 or br:
                    state["eobrun"] += 1
                    state["be"] += br
                    if state["eobrun"] == 0x7fff or len(state["be"]) > 937:
                        flush_eob()
        flush_eob()
        if emit:
            bw.flush()
        return dcf, acf, bw

    out = bytearray(b"\xff\xd8")
    if pad_ff:
        out += b"\xff"
    if jfif:
        out += b"\xff\xe0" + struct.pack(">H", 16) + b"JFIF\x00" + bytes([1, 1, 0, 0, 1, 0, 1, 0, 0])
    if adobe is not None:
        out += b"\xff\xee" + struct.pack(">H", 14) + b"Adobe\x00" + bytes([100, 0, 0, 0, 0, adobe])
    out += b"\xff\xfe" + struct.pack(">H", 2 + 9) + b"seeded!!!"
    for t in range(2):
        if dqt16:
            out += b"\xff\xdb" + struct.pack(">H", 2 + 129) + bytes([0x10 | t]) + \
                b"".join(struct.pack(">H", int(x)) for x in qt[t].reshape(64)[ZIGZAG])
        else:
            out += b"\xff\xdb" + struct.pack(">H", 2 + 65) + bytes([t]) + bytes(int(x) for x in qt[t].reshape(64)[ZIGZAG])
    sof = 0xc2 if progressive else (0xc1 if dqt16 else 0xc0)
    out += bytes([0xff, sof]) + struct.pack(">HBHHB", 8 + 3 * nc, 8, H, W, nc)
    for c in range(nc):
        out += bytes([ids[c], (samp[c][0] << 4) | samp[c][1], tq[c]])
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    for (comps, ss, se, ah, al) in scans:
        dcf, acf, _ = encode_scan(comps, ss, se, ah, al)
        dct = _huff_table(dcf) if dcf else None
        act = _huff_table(acf) if acf else None
        seg = bytearray()
        if dct:
            seg += bytes([0x00]) + bytes(dct[0]) + bytes(dct[1])
        if act:
            seg += bytes([0x10]) + bytes(act[0]) + bytes(act[1])
        if seg:
            out += b"\xff\xc4" + struct.pack(">H", 2 + len(seg)) + seg
        out += b"\xff\xda" + struct.pack(">HB", 6 + 2 * len(comps), len(comps))
        for c in comps:
            out += bytes([ids[c], 0x00])
        out += bytes([ss, se, (ah << 4) | al])
        tabs = ({k: v for k, v in dct[2].items()} if dct else {}, {k: v for k, v in act[2].items()} if act else {})
        _, _, bw = encode_scan(comps, ss, se, ah, al, tabs)
        out += bw.out
    out += b"\xff\xd9"
    return bytes(out)


def _smooth(rng, h, w):
    """A smooth seeded plane with some detail (uint8)."""
    y, x = np.mgrid[0:h, 0:w]
    v = 128 + 60 * np.sin(x / (2 + rng.uniform(0, 5)) + rng.uniform(0, 6)) * np.cos(y / (3 + rng.uniform(0, 5)))
    v += rng.normal(0, 12, (h, w))
    return np.clip(np.round(v), 0, 255).astype(np.uint8)


def jpeg_cases():
    rng = np.random.default_rng(15)
    cases = []

    def planes(W, H, samp):
        hmax = max(h for h, _ in samp)
        vmax = max(v for _, v in samp)
        return [_smooth(rng, -(-H * v // vmax), -(-W * h // hmax)) for h, v in samp]

    s444 = [(1, 1)] * 3
    s420 = [(2, 2), (1, 1), (1, 1)]
    s422 = [(2, 1), (1, 1), (1, 1)]
    s440 = [(1, 2), (1, 1), (1, 1)]
    s411 = [(4, 1), (1, 1), (1, 1)]
    cases.append(("gray.jpg", jpeg_bytes(planes(37, 29, [(1, 1)]), [(1, 1)])))
    cases.append(("ycc444.jpg", jpeg_bytes(planes(33, 21, s444), s444)))
    cases.append(("ycc420.jpg", jpeg_bytes(planes(45, 33, s420), s420, qscale=2.0)))
    cases.append(("ycc420_1px.jpg", jpeg_bytes(planes(1, 1, s420), s420)))
    cases.append(("ycc420_2x3.jpg", jpeg_bytes(planes(2, 3, s420), s420)))
    cases.append(("ycc422.jpg", jpeg_bytes(planes(40, 17, s422), s422)))
    cases.append(("ycc440.jpg", jpeg_bytes(planes(23, 40, s440), s440)))
    cases.append(("ycc411.jpg", jpeg_bytes(planes(50, 12, s411), s411)))
    cases.append(("ycc420_restart.jpg", jpeg_bytes(planes(70, 50, s420), s420, restart=3)))
    cases.append(("ycc420_planar.jpg", jpeg_bytes(planes(41, 35, s420), s420,
                                                 scans=[([0], 0, 63, 0, 0), ([1], 0, 63, 0, 0), ([2], 0, 63, 0, 0)])))
    cases.append(("ycc_dqt16.jpg", jpeg_bytes(planes(24, 18, s444), s444, qscale=0.5, dqt16=True)))
    cases.append(("rgb_ids.jpg", jpeg_bytes(planes(19, 13, s444), s444, ids=[ord("R"), ord("G"), ord("B")])))
    cases.append(("rgb_adobe.jpg", jpeg_bytes(planes(19, 13, s444), s444, adobe=0, jfif=False)))
    cases.append(("cmyk.jpg", jpeg_bytes(planes(21, 14, [(1, 1)] * 4), [(1, 1)] * 4, adobe=0, jfif=False)))
    cases.append(("ycck.jpg", jpeg_bytes(planes(21, 14, [(2, 2), (1, 1), (1, 1), (2, 2)]),
                                         [(2, 2), (1, 1), (1, 1), (2, 2)], adobe=2, jfif=False)))
    prog = [([0, 1, 2], 0, 0, 0, 1),
            ([0], 1, 5, 0, 2), ([2], 1, 63, 0, 1), ([1], 1, 63, 0, 1), ([0], 6, 63, 0, 2),
            ([0], 1, 63, 2, 1), ([0, 1, 2], 0, 0, 1, 0), ([2], 1, 63, 1, 0), ([1], 1, 63, 1, 0),
            ([0], 1, 63, 1, 0)]
    cases.append(("prog420.jpg", jpeg_bytes(planes(53, 37, s420), s420, scans=prog, progressive=True,
                                            qscale=0.7)))
    cases.append(("prog420_restart.jpg", jpeg_bytes(planes(53, 37, s420), s420, scans=prog, progressive=True,
                                                    restart=2, pad_ff=True)))
    cases.append(("prog_gray.jpg", jpeg_bytes(planes(30, 26, [(1, 1)]), [(1, 1)], progressive=True, qscale=0.4,
                                              scans=[([0], 0, 0, 0, 2), ([0], 1, 63, 0, 3), ([0], 0, 0, 2, 1),
                                                     ([0], 1, 63, 3, 2), ([0], 1, 63, 2, 1), ([0], 0, 0, 1, 0),
                                                     ([0], 1, 63, 1, 0)])))
    return cases


# ---------------------------------------------------------------------------
# BMP, TGA, GIF, PSD, Softimage PIC (small writers for the fixtures)
# ---------------------------------------------------------------------------
def bmp_bytes(img, bpp, hsz=40, top_down=False, compress=0, masks=None, palette=None):
    """img: (h, w, 3|4) uint8 for bpp >= 16, or (h, w) palette indices for
    bpp <= 8 (palette: (n, 3) RGB).  masks: (r, g, b[, a]) for compress 3 or
    the V4/V5 header's mask fields."""
    h, w = img.shape[:2]
    rows = []
    for y in range(h):
        if bpp == 24:
            row = img[y, :, 2::-1].tobytes()
        elif bpp == 32 and masks is None:
            px = img[y]
            a = px[:, 3] if px.shape[1] == 4 else np.zeros(w, np.uint8)
            row = np.stack([px[:, 2], px[:, 1], px[:, 0], a], 1).astype(np.uint8).tobytes()
        elif bpp in (16, 32):
            m = list(masks) + [0] * (4 - len(masks))
            vals = np.zeros(w, np.uint64)
            for c in range(4 if img.shape[2] == 4 else 3):
                mk = m[c]
                if not mk:
                    continue
                lo = (mk & -mk).bit_length() - 1
                nb = bin(mk).count("1")
                vals |= ((img[y, :, c].astype(np.uint64) >> np.uint64(8 - nb)) << np.uint64(lo))
            row = vals.astype("<u2" if bpp == 16 else "<u4").tobytes()
        elif bpp == 8:
            row = img[y].astype(np.uint8).tobytes()
        elif bpp == 4:
            v = list(img[y]) + ([0] if w % 2 else [])
            row = bytes((v[i] << 4) | v[i + 1] for i in range(0, len(v), 2))
        elif bpp == 1:
            v = list(img[y]) + [0] * ((-w) % 8)
            row = bytes(sum(v[i + k] << (7 - k) for k in range(8)) for i in range(0, len(v), 8))
        rows.append(row + b"\0" * ((-len(row)) % 4))
    if not top_down:
        rows = rows[::-1]
    data = b"".join(rows)
    pal = b""
    if palette is not None:
        for r, g, b in palette:
            pal += bytes([b, g, r]) + (b"" if hsz == 12 else b"\0")
    if hsz == 12:
        info = struct.pack("<IHHHH", 12, w, h, 1, bpp)
    else:
        hh = -h if top_down else h
        info = struct.pack("<IiiHHIIiiII", hsz, w, hh, 1, bpp, compress, len(data), 2835, 2835, 0, 0)
        if hsz == 40 and compress == 3:
            info += struct.pack("<III", *masks[:3])
        elif hsz == 56:
            info += struct.pack("<IIII", *(list(masks or [0, 0, 0, 0]) + [0] * 4)[:4])
        elif hsz in (108, 124):
            info += struct.pack("<IIII", *(list(masks or [0, 0, 0, 0]) + [0] * 4)[:4])
            info += struct.pack("<I", 0x73524742) + b"\0" * 48
            if hsz == 124:
                info += b"\0" * 16
    offset = 14 + len(info) + len(pal)
    head = b"BM" + struct.pack("<IHHI", offset + len(data), 0, 0, offset)
    return head + info + pal + data


def bmp_cases():
    rng = np.random.default_rng(21)
    rgb = rng.integers(0, 256, (7, 13, 3), np.uint8)
    rgba = rng.integers(0, 256, (6, 9, 4), np.uint8)
    zero_a = rgba.copy()
    zero_a[..., 3] = 0
    pal = rng.integers(0, 256, (256, 3), np.uint8)
    idx8 = rng.integers(0, 256, (5, 11), np.uint8)
    idx4 = rng.integers(0, 16, (6, 9), np.uint8)
    idx1 = rng.integers(0, 2, (4, 19), np.uint8)
    os2_idx = rng.integers(0, 200, (5, 6), np.uint8)  # the OS/2 palette size formula reads 4 entries fewer
    return [("rgb24.bmp", bmp_bytes(rgb, 24)),
            ("rgb24_topdown.bmp", bmp_bytes(rgb, 24, top_down=True)),
            ("rgba32_bi_rgb.bmp", bmp_bytes(rgba, 32)),
            ("rgba32_v4.bmp", bmp_bytes(rgba, 32, hsz=108)),
            ("rgba32_v5_zero_alpha.bmp", bmp_bytes(zero_a, 32, hsz=124, top_down=True)),
            ("rgb32_bitfields.bmp", bmp_bytes(rgba[..., :3], 32, compress=3,
                                              masks=(0xff000000, 0x00ff0000, 0x0000ff00))),
            ("rgb16_555.bmp", bmp_bytes(rgb, 16, masks=(0x7c00, 0x03e0, 0x001f))),
            ("rgb16_565.bmp", bmp_bytes(rgb, 16, compress=3, masks=(0xf800, 0x07e0, 0x001f))),
            ("rgba16_4444_v4.bmp", bmp_bytes(rgba, 16, hsz=108, compress=3,
                                             masks=(0x0f00, 0x00f0, 0x000f, 0xf000))),
            ("pal8.bmp", bmp_bytes(idx8, 8, palette=pal)),
            ("pal4.bmp", bmp_bytes(idx4, 4, palette=pal[:16])),
            ("pal1.bmp", bmp_bytes(idx1, 1, palette=pal[:2])),
            ("os2_rgb24.bmp", bmp_bytes(rgb, 24, hsz=12)),
            ("os2_pal8.bmp", bmp_bytes(os2_idx, 8, hsz=12, palette=pal))]


def _tga_rle(pixels):
    """pixels: list of byte strings; run-length packets (runs of >= 2)."""
    out, i, n = [], 0, len(pixels)
    while i < n:
        j = i
        while j + 1 < n and pixels[j + 1] == pixels[i] and j - i < 127:
            j += 1
        if j > i:
            out.append(bytes([0x80 | (j - i)]) + pixels[i])
            i = j + 1
            continue
        j = i
        while j + 1 < n and pixels[j + 1] != pixels[j] and j - i < 127:
            j += 1
        out.append(bytes([j - i]) + b"".join(pixels[i:j + 1]))
        i = j + 1
    return b"".join(out)


def tga_bytes(pix, image_type, bpp, top_down=False, palette=None, pal_bits=0, image_id=b""):
    """pix: (h, w, c) raw pixel bytes in file order (B, G, R[, A]), or (h, w)
    indices / grey; palette: (n, pal_bits / 8) entry bytes in file order."""
    h, w = pix.shape[:2]
    rows = [pix[y] for y in range(h)]
    if not top_down:
        rows = rows[::-1]
    bpx = bpp // 8 if bpp != 15 else 2
    flat = []
    for row in rows:
        if row.ndim == 1:
            if bpx == 2:
                flat += [struct.pack("<H", int(v)) for v in row]
            else:
                flat += [bytes([int(v)]) for v in row]
        else:
            flat += [row[x].astype(np.uint8).tobytes() for x in range(w)]
    data = _tga_rle(flat) if image_type >= 8 else b"".join(flat)
    cmap = 1 if palette is not None else 0
    n_pal = 0 if palette is None else len(palette)
    head = struct.pack("<BBBHHBHHHHBB", len(image_id), cmap, image_type, 0, n_pal, pal_bits, 0, 0, w, h, bpp,
                       0x20 if top_down else 0)
    pal = b"" if palette is None else np.asarray(palette, np.uint8).tobytes()
    return head + image_id + pal + data


def tga_cases():
    rng = np.random.default_rng(22)
    bgr = rng.integers(0, 256, (6, 7, 3), np.uint8)
    bgra = rng.integers(0, 256, (5, 8, 4), np.uint8)
    grey = rng.integers(0, 256, (4, 9), np.uint8)
    ga = rng.integers(0, 256, (5, 6, 2), np.uint8)
    # images with runs for the RLE forms (runs cross row ends)
    runs = rng.integers(0, 4, (9, 10), np.uint8)
    run_cols = rng.integers(0, 256, (4, 3), np.uint8)
    bgr_runs = run_cols[runs]
    grey_runs = (runs * 60).astype(np.uint8)
    pal24 = rng.integers(0, 256, (40, 3), np.uint8)
    pal32 = rng.integers(0, 256, (16, 4), np.uint8)
    pal16 = rng.integers(0, 1 << 15, 20).astype("<u2").view(np.uint8).reshape(20, 2)
    idx = rng.integers(0, 40, (6, 5), np.uint8)
    idx_bad = idx.copy()
    idx_bad[0, 0] = 250  # out of the palette: entry 0
    c16 = rng.integers(0, 1 << 15, (4, 5)).astype(np.uint16)
    return [("bgr24.tga", tga_bytes(bgr, 2, 24)),
            ("bgra32_topdown.tga", tga_bytes(bgra, 2, 32, top_down=True, image_id=b"kagayaki")),
            ("grey8.tga", tga_bytes(grey, 3, 8)),
            ("grey_alpha16.tga", tga_bytes(ga, 3, 16, top_down=True)),
            ("rgb15.tga", tga_bytes(c16, 2, 16)),
            ("rle_bgr24.tga", tga_bytes(bgr_runs, 10, 24)),
            ("rle_grey8.tga", tga_bytes(grey_runs, 11, 8, top_down=True)),
            ("pal24.tga", tga_bytes(idx_bad, 1, 8, palette=pal24, pal_bits=24)),
            ("rle_pal32.tga", tga_bytes((runs * 3).astype(np.uint8), 9, 8, palette=pal32, pal_bits=32)),
            ("pal16.tga", tga_bytes((idx % 20).astype(np.uint8), 1, 8, palette=pal16, pal_bits=16))]


def _lzw_codes(indices, min_size):
    """GIF LZW codes with the widths a reader uses: (code, width) pairs."""
    clear, end = 1 << min_size, (1 << min_size) + 1
    out = []
    size = min_size + 1
    table, nxt, avail, k = {}, clear + 2, clear + 2, 0

    def reset():
        nonlocal table, nxt, avail, size, k
        table = {(i,): i for i in range(clear)}
        nxt, avail, size, k = clear + 2, clear + 2, min_size + 1, 0

    def emit(code):
        nonlocal avail, size, k
        out.append((code, size))
        k += 1
        if k >= 2:  # the reader adds an entry for every code after the first
            avail += 1
            if (avail & ((1 << size) - 1)) == 0 and avail <= 0xfff:
                size += 1

    out.append((clear, size))
    reset()
    w = ()
    for c in indices:
        wc = w + (int(c),)
        if wc in table:
            w = wc
            continue
        emit(table[w])
        table[wc] = nxt
        nxt += 1
        w = (int(c),)
        if nxt >= 4000:
            emit(table[w])
            w = ()
            out.append((clear, size))
            reset()
    if w:
        emit(table[w])
    out.append((end, size))
    return out


def _gif_raster(indices, min_size):
    acc = nbits = 0
    data = bytearray()
    for code, width in _lzw_codes(indices, min_size):
        acc |= code << nbits
        nbits += width
        while nbits >= 8:
            data.append(acc & 0xff)
            acc >>= 8
            nbits -= 8
    if nbits:
        data.append(acc & 0xff)
    blocks = b"".join(bytes([len(data[i:i + 255])]) + bytes(data[i:i + 255]) for i in range(0, len(data), 255))
    return bytes([min_size]) + blocks + b"\0"


def gif_bytes(W, H, gpal=None, bg=0, frame=None, gce=None, exts=()):
    """frame: (x, y, idx (h, w), lpal or None, interlaced)."""
    def table_bits(pal):
        n = 2
        k = 0
        while n < len(pal):
            n *= 2
            k += 1
        return k, n

    out = b"GIF89a" + struct.pack("<HH", W, H)
    if gpal is not None:
        k, n = table_bits(gpal)
        out += bytes([0x80 | k, bg, 0])
        out += np.asarray(gpal, np.uint8).tobytes() + b"\0" * (3 * (n - len(gpal)))
    else:
        out += bytes([0, bg, 0])
    for e in exts:
        out += e
    if gce is not None:  # (transparent index or None)
        out += b"\x21\xf9\x04" + bytes([1 if gce[0] is not None else 0]) + b"\0\0" + \
            bytes([gce[0] or 0]) + b"\0"
    x, y, idx, lpal, interlaced = frame
    h, w = idx.shape
    flags = 0x40 if interlaced else 0
    pal_used = gpal
    if lpal is not None:
        k, n = table_bits(lpal)
        flags |= 0x80 | k
        pal_used = lpal
    out += b"\x2c" + struct.pack("<HHHH", x, y, w, h) + bytes([flags])
    if lpal is not None:
        out += np.asarray(lpal, np.uint8).tobytes() + b"\0" * (3 * (n - len(lpal)))
    rows = list(range(h))
    if interlaced:
        rows = list(range(0, h, 8)) + list(range(4, h, 8)) + list(range(2, h, 4)) + list(range(1, h, 2))
    seq = np.concatenate([idx[r] for r in rows])
    min_size = max(2, int(np.ceil(np.log2(max(len(pal_used), 2)))))
    return out + _gif_raster(seq, min_size) + b"\x3b"


def gif_cases():
    rng = np.random.default_rng(23)
    pal = rng.integers(0, 256, (256, 3), np.uint8)
    noisy = rng.integers(0, 256, (70, 64), np.uint8)  # the code table fills and restarts
    smooth = (np.add.outer(np.arange(21), np.arange(17)) // 3 % 16).astype(np.uint8)
    two = rng.integers(0, 2, (9, 14), np.uint8)
    comment = b"\x21\xfe\x05hello\x00"
    app = b"\x21\xff\x0bNETSCAPE2.0\x03\x01\x00\x00\x00"
    return [("noisy256.gif", gif_bytes(64, 70, pal, frame=(0, 0, noisy, None, False))),
            ("interlaced.gif", gif_bytes(17, 21, pal[:16], frame=(0, 0, smooth, None, True), exts=(comment,))),
            ("local_transparent.gif", gif_bytes(17, 21, None, frame=(0, 0, smooth, pal[16:32], False),
                                                gce=(5,), exts=(app,))),
            ("sub_frame_bg.gif", gif_bytes(20, 15, pal[:32], bg=7, frame=(3, 2, smooth[:9, :11] + 8, None, False),
                                           gce=(9,))),
            ("two_colour.gif", gif_bytes(14, 9, pal[100:102], frame=(0, 0, two, None, False)))]


def _psd_rle_row(row):
    out, i, n = bytearray(), 0, len(row)
    while i < n:
        j = i
        while j + 1 < n and row[j + 1] == row[i] and j - i < 127:
            j += 1
        if j > i:
            out += bytes([257 - (j - i + 1), row[i]])
            i = j + 1
            continue
        j = i
        while j + 1 < n and row[j + 1] != row[j] and j - i < 127:
            j += 1
        out += bytes([j - i]) + bytes(row[i:j + 1])
        i = j + 1
    return bytes(out)


def psd_bytes(planes, depth=8, rle=False):
    """planes: (c, h, w) channel planes (uint8, or uint16 for depth 16)."""
    c, h, w = planes.shape
    head = b"8BPS" + struct.pack(">H", 1) + b"\0" * 6 + struct.pack(">HIIHH", c, h, w, depth, 3)
    head += struct.pack(">I", 0) + struct.pack(">I", 6) + b"\0" * 6 + struct.pack(">I", 0)
    if not rle:
        body = planes.astype(">u2" if depth == 16 else np.uint8).tobytes()
        return head + struct.pack(">H", 0) + body
    rows = [_psd_rle_row(bytes(planes[k, y].astype(np.uint8))) for k in range(c) for y in range(h)]
    counts = b"".join(struct.pack(">H", len(r)) for r in rows)
    return head + struct.pack(">H", 1) + counts + b"".join(rows)


def psd_cases():
    rng = np.random.default_rng(24)
    rgb = rng.integers(0, 256, (3, 5, 7), np.uint8)
    rgba = rng.integers(0, 256, (4, 6, 5), np.uint8)
    rgba[3, 0, :3] = [0, 255, 128]
    runs = rng.integers(0, 3, (5, 6, 40)).astype(np.uint8) * 80
    deep = rng.integers(0, 65536, (4, 3, 4)).astype(np.uint16)
    one = rng.integers(0, 256, (1, 4, 4), np.uint8)
    return [("rgb8.psd", psd_bytes(rgb)),
            ("rgba8_matte.psd", psd_bytes(rgba)),
            ("rle5.psd", psd_bytes(runs, rle=True)),
            ("rgba16.psd", psd_bytes(deep, depth=16)),
            ("one_channel.psd", psd_bytes(one))]


def pic_bytes(img, packets):
    """img: (h, w, 4) RGBA; packets: [(channel mask, type)], chained in order.
    Types: 0 raw, 1 pure run-length, 2 mixed run-length."""
    h, w = img.shape[:2]
    head = bytes([0x53, 0x80, 0xF6, 0x34]) + struct.pack(">f", 3.71) + b"kagayaki".ljust(80, b"\0") + b"PICT"
    head += struct.pack(">HHfHH", w, h, 1.0, 3, 0)
    for i, (ch, t) in enumerate(packets):
        head += bytes([1 if i + 1 < len(packets) else 0, 8, t, ch])
    sel = lambda ch: [k for k in range(4) if ch & (0x80 >> k)]  # noqa: E731
    body = bytearray()
    for y in range(h):
        for ch, t in packets:
            ks = sel(ch)
            vals = [bytes(img[y, x, ks]) for x in range(w)]
            if t == 0:
                body += b"".join(vals)
            elif t == 1:
                x = 0
                while x < w:
                    n = 1
                    while x + n < w and vals[x + n] == vals[x] and n < 255:
                        n += 1
                    body += bytes([n]) + vals[x]
                    x += n
            else:
                x = 0
                while x < w:
                    n = 1
                    while x + n < w and vals[x + n] == vals[x] and n < 300:
                        n += 1
                    if n >= 2:
                        body += (bytes([n + 127]) if n <= 127 else b"\x80" + struct.pack(">H", n)) + vals[x]
                        x += n
                    else:
                        m = 1
                        while x + m < w and m < 128 and (x + m + 1 >= w or vals[x + m + 1] != vals[x + m]):
                            m += 1
                        body += bytes([m - 1]) + b"".join(vals[x:x + m])
                        x += m
    return head + bytes(body)


def pic_cases():
    rng = np.random.default_rng(25)
    img = rng.integers(0, 256, (5, 9, 4), np.uint8)
    runs = (rng.integers(0, 3, (6, 150, 4)) * 100).astype(np.uint8)
    runs[:, :140] = runs[:, :1]  # long runs: the 16-bit count form
    return [("raw_rgb.pic", pic_bytes(img, [(0xE0, 0)])),
            ("pure_rle_rgba.pic", pic_bytes(runs[:, :20], [(0xE0, 1), (0x10, 1)])),
            ("mixed_rle_rgba.pic", pic_bytes(runs, [(0xF0, 2)])),
            ("split_channels.pic", pic_bytes(img, [(0x80, 0), (0x60, 2), (0x10, 1)]))]


def image_cases():
    return png_cases() + hdr_cases() + pnm_cases() + jpeg_cases() + bmp_cases() + tga_cases() + gif_cases() + \
        psd_cases() + pic_cases()


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
usemtl tex_jpg
f 10/2/5 12/4/5 14/1/5
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

newmtl tex_jpg
map_Kd tex_jpg.jpg
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
    with open(os.path.join(d, "tex_jpg.jpg"), "wb") as f:
        s420 = [(2, 2), (1, 1), (1, 1)]
        f.write(jpeg_bytes([_smooth(rng, 14, 22), _smooth(rng, 7, 11), _smooth(rng, 7, 11)], s420))
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
