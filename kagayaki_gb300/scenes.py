"""Seeded procedural scenes and ray sets.

Every random draw comes from SplitMix64 counters in uint64 arithmetic and
every float is produced by correctly rounded operations (+ - * / sqrt), so the
same seed gives the same bytes on x86 and Arm.  Transcendentals (sin, cos, exp)
appear only in inputs that are generated once per process and fed to both the
GPU path and the oracle (mesh noise, environment texels), never in golden
fixtures.

Scenes:
  cornell_box()        - 36 triangles: 5 walls, two boxes rotated +-18 deg, a
                         2-triangle emissive ceiling light (17,12,4); Lambert.
  icosphere_field()    - N displaced icospheres (subdivision s) over a ground
                         quad; Disney materials drawn per mesh; z up.
  c5_scene()           - 128 icospheres on a 256 x 256-tile heightfield with
                         64 procedural RGBA8 textures (10.6 M triangles).
  sky_environment()    - lat-long float32 RGB environment in the reference's
                         mapping (ImageBasedLighting.cuh:6-56): sky gradient and
                         a sun lobe of a given peak radiance.
  parity_rays()        - origins uniform in a box, directions uniform on the
                         sphere (rejection from the unit ball).
"""
import numpy as np

from .structs import DISNEY, LAMBERT, MATERIAL, RAY, TRIANGLE, make_material

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x):
    """SplitMix64 finaliser of a uint64 array (wrapping arithmetic)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def xorshift64(s):
    """The reference's 64-bit xorshift step, shifts 5/41/20
    (struct_Xorshift.cuh:10-20)."""
    s = np.asarray(s, dtype=np.uint64)
    with np.errstate(over="ignore"):
        s = s ^ (s << np.uint64(5))
        s = s ^ (s >> np.uint64(41))
        s = s ^ (s << np.uint64(20))
    return s


class CounterRng:
    """Uniform doubles in [0,1) from SplitMix64(seed, counter)."""

    def __init__(self, seed):
        self.key = splitmix64(np.uint64(seed) ^ np.uint64(0x5EED5EED5EED5EED))
        self.ctr = 0

    def uniform(self, n, lo=0.0, hi=1.0):
        idx = np.arange(self.ctr, self.ctr + n, dtype=np.uint64)
        self.ctr += n
        with np.errstate(over="ignore"):
            bits = splitmix64(self.key + idx * np.uint64(0xD1B54A32D192ED03))
        u = (bits >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u


# --------------------------------------------------------------------------
# Triangle assembly helpers
# --------------------------------------------------------------------------

def canonical(tris):
    """Copy of TRIANGLE records with the C padding bytes zeroed (numpy copies
    may leave arbitrary bytes there), so byte digests are reproducible."""
    out = np.zeros(len(tris), dtype=TRIANGLE)
    for f in TRIANGLE.names:
        out[f] = tris[f]
    return out


def _tris_from_indexed(pos, nrm, uv, faces, material_id, smooth, shape_id):
    """Indexed mesh -> TRIANGLE records (positions/normals/uvs per vertex)."""
    n = len(faces)
    t = np.zeros(n, dtype=TRIANGLE)
    v = t["verts"]
    for k in range(3):
        v[:, k, :3] = pos[faces[:, k]]
        v[:, 3 + k, :3] = nrm[faces[:, k]]
        v[:, 6 + k, :2] = uv[faces[:, k]]
    t["material_id"] = material_id
    t["is_SmoothNormal"] = 1 if smooth else 0
    t["shape_id"] = shape_id
    return t


def _quad(p0, p1, p2, p3, material_id, shape_id):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with flat vertex normals."""
    pos = np.array([p0, p1, p2, p3], dtype=np.float64)
    n = np.cross(pos[1] - pos[0], pos[2] - pos[0])
    n = n / np.sqrt((n * n).sum())
    nrm = np.repeat(n[None, :], 4, axis=0)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float64)
    faces = np.array([[0, 1, 2], [0, 2, 3]])
    return _tris_from_indexed(pos.astype(np.float32), nrm.astype(np.float32),
                              uv.astype(np.float32), faces, material_id, False, shape_id)


def _box(center_xz, size, height, y0, angle_deg, material_id, shape_id):
    """Axis-aligned box rotated about +y: 6 quads = 12 triangles, outward
    normals.  The rotation uses a fixed sin/cos pair rounded to float32."""
    a = np.deg2rad(angle_deg)
    c, s = np.float32(np.cos(a)), np.float32(np.sin(a))
    hx = size / 2.0
    corners = []
    for yy in (y0, y0 + height):
        for (x, z) in ((-hx, -hx), (hx, -hx), (hx, hx), (-hx, hx)):
            rx = c * x + s * z + center_xz[0]
            rz = -s * x + c * z + center_xz[1]
            corners.append((rx, yy, rz))
    b = corners
    quads = [(b[0], b[1], b[2], b[3]),  # bottom (normal -y)
             (b[4], b[7], b[6], b[5]),  # top (+y)
             (b[0], b[4], b[5], b[1]),  # side
             (b[1], b[5], b[6], b[2]),
             (b[2], b[6], b[7], b[3]),
             (b[3], b[7], b[4], b[0])]
    return np.concatenate([_quad(*q, material_id, shape_id) for q in quads])


# --------------------------------------------------------------------------
# Config 1: Cornell-style box
# --------------------------------------------------------------------------

CORNELL_LO = (-5.0, 0.0, -5.0)
CORNELL_HI = (5.0, 10.0, 5.0)


def cornell_box():
    """Returns (triangles, materials, camera_args).

    Box [-5,5] x [0,10] x [-5,5], open toward +z.  Materials: 0 grey 0.73,
    1 red (0.63,0.065,0.05), 2 green (0.14,0.45,0.09), 3 light (emission
    (17,12,4)).  The light quad sits 1e-3 under the ceiling and the boxes 1e-3
    above the floor, so no two faces are coplanar.
    """
    mats = np.stack([
        make_material(LAMBERT, (0.73, 0.73, 0.73)),
        make_material(LAMBERT, (0.63, 0.065, 0.05)),
        make_material(LAMBERT, (0.14, 0.45, 0.09)),
        make_material(LAMBERT, (0.78, 0.78, 0.78), emission=(17.0, 12.0, 4.0)),
    ])
    x0, y0, z0 = CORNELL_LO
    x1, y1, z1 = CORNELL_HI
    parts = [
        _quad((x0, y0, z1), (x1, y0, z1), (x1, y0, z0), (x0, y0, z0), 0, 0),  # floor
        _quad((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1), 0, 1),  # ceiling
        _quad((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0), 0, 2),  # back
        _quad((x0, y0, z1), (x0, y0, z0), (x0, y1, z0), (x0, y1, z1), 1, 3),  # left
        _quad((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0), 2, 4),  # right
        _box((1.8, 1.2), 3.0, 3.0, 1e-3, -18.0, 0, 5),                         # short box
        _box((-1.8, -1.6), 3.0, 6.0, 1e-3, 18.0, 0, 6),                        # tall box
    ]
    ly = y1 - 1e-3
    parts.append(_quad((-1.25, ly, -1.25), (1.25, ly, -1.25), (1.25, ly, 1.25),
                       (-1.25, ly, 1.25), 3, 7))
    tris = canonical(np.concatenate(parts))
    assert len(tris) == 36
    cam = dict(origin=(0.0173, 5.0131, 13.6), dist=28.0, rot=(0.0, 0.0, 0.0))
    return tris, mats, cam


def parity_scene(kind):
    """Small seeded scenes on which the reference's own estimator is compared
    sample for sample with the reference's render.  Returns (triangles,
    materials, camera args (origin, dist, rot), textures (list of (h, w, bpp)
    float32 arrays, indexed by TEXTURE_BASECOLOR_ID), environment or None).

      cornell   cornell_box() as it is: Lambert walls and boxes, a face light
      disney    the same box with Disney boxes: the short one a rough metal,
                the tall one a clearcoated dielectric with sheen, sheen tint,
                specular tint and anisotropy
      textured  the same box with a textured back wall (RGB, 64 x 48) and
                floor (RGBA, 32 x 32), seeded; their uvs stay inside
                [0.02, 0.98], where the reference's nearest fetch
                (struct_Texture.cuh:12-18) reads inside the texel array
      env       two displaced Disney icospheres (1,280 triangles each) over a
                ground quad under a 64 x 32 float32 sky with a sun lobe of
                peak 100, no face light
    """
    if kind == "env":
        tris, mats, info = icosphere_field(n_meshes=2, subdiv=3, seed=5, box=6.0)
        env, _ = sky_environment(64, 32, sun_peak=100.0, seed=3)
        ang, radius, z, tz = 37.0, 12.0, 4.0, 2.5
        a = np.deg2rad(ang)
        org = (radius * np.cos(a), radius * np.sin(a), z)
        pitch = np.rad2deg(np.arctan2(z - tz, radius))
        cam = dict(origin=org, dist=28.0, rot=(90.0 - pitch, 0.0, ang + 90.0))
        return tris, mats, cam, [], np.ascontiguousarray(env, np.float32)
    tris, mats, cam = cornell_box()
    tris = tris.copy()
    textures = []
    if kind == "disney":
        metal = make_material(DISNEY, (0.9, 0.62, 0.3), metallic=1.0, roughness=0.35, specular=0.5)
        coat = make_material(DISNEY, (0.2, 0.35, 0.75), roughness=0.6, specular=0.5, specularTint=0.4,
                             sheen=0.7, sheenTint=0.5, clearcoat=0.8, cloearcoatGloss=0.7, anisotropic=0.4)
        mats = np.concatenate([mats, np.stack([metal, coat])])
        tris["material_id"][tris["shape_id"] == 5] = len(mats) - 2
        tris["material_id"][tris["shape_id"] == 6] = len(mats) - 1
    elif kind == "textured":
        rng = CounterRng(17)
        wall = rng.uniform(48 * 64 * 3, 0.05, 0.95).reshape(48, 64, 3).astype(np.float32)
        floor = rng.uniform(32 * 32 * 4, 0.05, 0.95).reshape(32, 32, 4).astype(np.float32)
        textures = [wall, floor]
        mats = np.concatenate([mats, np.stack([make_material(LAMBERT, (0.8, 0.8, 0.8)),
                                               make_material(LAMBERT, (0.8, 0.8, 0.8))])])
        mats["TEXTURE_BASECOLOR_ID"][-2:] = (0, 1)
        for shape, mat in ((2, len(mats) - 2), (0, len(mats) - 1)):  # back wall, floor
            sel = tris["shape_id"] == shape
            tris["material_id"][sel] = mat
            uv = tris["verts"][sel, 6:9, :2]
            tris["verts"][sel, 6:9, :2] = 0.02 + 0.96 * uv
    elif kind != "cornell":
        raise ValueError(f"unknown parity scene {kind!r}")
    return canonical(tris), mats, cam, textures, None


# --------------------------------------------------------------------------
# Config 2: displaced icosphere field
# --------------------------------------------------------------------------

def icosphere(subdiv):
    """Unit icosphere: (vertices float64 (V,3), faces int32 (F,3)),
    F = 20 * 4**subdiv."""
    t = (1.0 + np.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.sqrt((v * v).sum(1, keepdims=True))
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.sqrt((mid * mid).sum(1, keepdims=True))
        mid_idx = inv + len(v)
        nf = len(f)
        m01, m12, m20 = mid_idx[:nf], mid_idx[nf:2 * nf], mid_idx[2 * nf:]
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f.astype(np.int32)


def _lattice_hash(ix, iy, iz, seed):
    """Integer lattice hash -> value in [-1, 1]."""
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343)
             ^ iy.astype(np.uint64) * np.uint64(0xD8163841)
             ^ iz.astype(np.uint64) * np.uint64(0xCB1AB31F)
             ^ np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15))
        h = splitmix64(h)
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def value_noise3(p, seed, octaves=3):
    """Sum of `octaves` trilinear value-noise octaves (freq 2^k * 2, amplitude
    0.5^k), normalised to [-1, 1]."""
    total = np.zeros(len(p))
    norm = 0.0
    for k in range(octaves):
        freq = 2.0 * (2 ** k)
        amp = 0.5 ** k
        q = p * freq + 1000.0
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        f = f * f * (3.0 - 2.0 * f)
        acc = np.zeros(len(p))
        for dx in (0, 1):
            wx = f[:, 0] if dx else 1.0 - f[:, 0]
            for dy in (0, 1):
                wy = f[:, 1] if dy else 1.0 - f[:, 1]
                for dz in (0, 1):
                    wz = f[:, 2] if dz else 1.0 - f[:, 2]
                    acc += wx * wy * wz * _lattice_hash(i0[:, 0] + dx, i0[:, 1] + dy,
                                                        i0[:, 2] + dz, seed * 131 + k)
        total += amp * acc
        norm += amp
    return total / norm


def icosphere_field(n_meshes=64, subdiv=6, seed=2, box=20.0, amplitude=0.05,
                    ground_half=100.0):
    """Config-2 style scene.  Returns (triangles, materials, info dict).

    n_meshes icospheres of 20*4**subdiv triangles, vertices displaced along
    the normal by amplitude*radius*noise (3-octave value noise), centres
    uniform in [-box/2, box/2]^2 x [r, box] (z up), radii uniform in
    [0.75, 2.0], over a 2-triangle ground quad at z = 0.  Material 0 is the
    ground (Disney grey); material 1+i belongs to mesh i with baseColor
    U[0.05,0.95]^3, metallic 1 with p = 0.3, roughness U[0.05,1],
    specular 0.5, clearcoat U[0,1].
    """
    rng = CounterRng(seed)
    base_v, base_f = icosphere(subdiv)
    nv = len(base_v)
    radii = rng.uniform(n_meshes, 0.75, 2.0)
    cx = rng.uniform(n_meshes, -box / 2, box / 2)
    cy = rng.uniform(n_meshes, -box / 2, box / 2)
    cz = radii + rng.uniform(n_meshes) * (box - radii)
    mats = [make_material(DISNEY, (0.5, 0.5, 0.5), roughness=0.6, specular=0.5)]
    for i in range(n_meshes):
        col = rng.uniform(3, 0.05, 0.95)
        metallic = 1.0 if rng.uniform(1)[0] < 0.3 else 0.0
        rough = rng.uniform(1, 0.05, 1.0)[0]
        coat = rng.uniform(1)[0]
        mats.append(make_material(DISNEY, tuple(col), metallic=metallic, roughness=rough,
                                  specular=0.5, clearcoat=coat))
    mats = np.stack(mats)

    uv = np.stack([np.arctan2(base_v[:, 1], base_v[:, 0]) / (2 * np.pi) + 0.5,
                   np.arccos(np.clip(base_v[:, 2], -1, 1)) / np.pi], 1).astype(np.float32)
    parts = []
    for i in range(n_meshes):
        disp = 1.0 + amplitude * value_noise3(base_v, seed * 1000 + i)
        pos = base_v * (radii[i] * disp)[:, None] + np.array([cx[i], cy[i], cz[i]])
        fn = np.cross(pos[base_f[:, 1]] - pos[base_f[:, 0]], pos[base_f[:, 2]] - pos[base_f[:, 0]])
        vn = np.zeros((nv, 3))
        for k in range(3):
            for c in range(3):
                vn[:, c] += np.bincount(base_f[:, k], weights=fn[:, c], minlength=nv)
        vn /= np.sqrt((vn * vn).sum(1, keepdims=True))
        parts.append(_tris_from_indexed(pos.astype(np.float32), vn.astype(np.float32), uv,
                                        base_f, 1 + i, True, i))
    g = ground_half
    parts.append(_quad((-g, -g, 0.0), (g, -g, 0.0), (g, g, 0.0), (-g, g, 0.0), 0, n_meshes))
    tris = canonical(np.concatenate(parts))
    info = dict(centers=np.stack([cx, cy, cz], 1), radii=radii,
                lo=(-box / 2, -box / 2, 0.0), hi=(box / 2, box / 2, box))
    return tris, mats, info


def value_noise2(x, y, seed, octaves=3, base_freq=4.0):
    """2D value noise over arrays x, y in [0, 1): `octaves` bilinear octaves
    (freq base_freq * 2^k, amplitude 0.5^k), smoothstep-interpolated,
    normalised to [-1, 1].  The lattice points' hashes are computed once and
    gathered; on a grid (x constant down columns, y along rows) the x
    interpolation runs once per lattice row - the same operations on the same
    values, so the same result."""
    x, y = np.broadcast_arrays(np.asarray(x, np.float64), np.asarray(y, np.float64))
    grid = x.ndim == 2 and bool((x == x[:1]).all()) and bool((y == y[:, :1]).all())
    total = np.zeros(x.shape)
    norm = 0.0
    for k in range(octaves):
        freq = base_freq * (2 ** k)
        amp = 0.5 ** k
        qx, qy = (x[0], y[:, 0]) if grid else (x, y)
        qx, qy = qx * freq + 1000.0, qy * freq + 1000.0
        ix, iy = np.floor(qx).astype(np.int64), np.floor(qy).astype(np.int64)
        fx, fy = qx - ix, qy - iy
        fx, fy = fx * fx * (3.0 - 2.0 * fx), fy * fy * (3.0 - 2.0 * fy)
        x0, y0 = int(ix.min()), int(iy.min())
        nx, ny = int(ix.max()) - x0 + 2, int(iy.max()) - y0 + 2
        if grid:
            gy, gx = np.mgrid[y0:y0 + ny, x0:x0 + nx]
            T = _lattice_hash(gx, gy, np.zeros_like(gx), seed * 131 + k)
            jx, jy = ix - x0, iy - y0
            B = T[:, jx] * (1 - fx) + T[:, jx + 1] * fx  # lattice rows interpolated in x
            total += amp * (B[jy] * (1 - fy)[:, None] + B[jy + 1] * fy[:, None])
        else:
            if nx * ny <= ix.size:
                gy, gx = np.mgrid[y0:y0 + ny, x0:x0 + nx]
                T = _lattice_hash(gx, gy, np.zeros_like(gx), seed * 131 + k)
                jx, jy = ix - x0, iy - y0
                h00, h10, h01, h11 = T[jy, jx], T[jy, jx + 1], T[jy + 1, jx], T[jy + 1, jx + 1]
            else:
                z = np.zeros_like(ix)
                h00 = _lattice_hash(ix, iy, z, seed * 131 + k)
                h10 = _lattice_hash(ix + 1, iy, z, seed * 131 + k)
                h01 = _lattice_hash(ix, iy + 1, z, seed * 131 + k)
                h11 = _lattice_hash(ix + 1, iy + 1, z, seed * 131 + k)
            total += amp * ((h00 * (1 - fx) + h10 * fx) * (1 - fy) + (h01 * (1 - fx) + h11 * fx) * fy)
        norm += amp
    return total / norm


def heightfield_terrain(tiles=256, half=150.0, height=6.0, seed=9, material_id=0, shape_id=0, uv_repeat=8.0):
    """A tiles x tiles grid of quads (2 * tiles^2 triangles) over
    [-half, half]^2 at z = height * noise (3-octave value noise), smooth
    normals, uv repeating uv_repeat times across the terrain."""
    n = tiles + 1
    g = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(g, g, indexing="xy")
    Z = height * value_noise2(X, Y, seed, octaves=4, base_freq=3.0)
    pos = np.stack([(X * 2 - 1) * half, (Y * 2 - 1) * half, Z], -1).reshape(-1, 3)
    uv = np.stack([X * uv_repeat, Y * uv_repeat], -1).reshape(-1, 2).astype(np.float32)
    i = np.arange(tiles)
    I, J = np.meshgrid(i, i, indexing="xy")
    v00 = (J * n + I).reshape(-1)
    v10, v01, v11 = v00 + 1, v00 + n, v00 + n + 1
    faces = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)]).astype(np.int64)
    fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        for c in range(3):
            vn[:, c] += np.bincount(faces[:, k], weights=fn[:, c], minlength=len(pos))
    vn /= np.sqrt((vn * vn).sum(1, keepdims=True))
    return _tris_from_indexed(pos.astype(np.float32), vn.astype(np.float32), uv, faces, material_id, True,
                              shape_id)


def procedural_textures_rgba8(n=64, size=1024, seed=21):
    """n seeded RGBA8 textures (size x size): per texture a checker of a random
    period blended with value noise between two random colours."""
    rng = CounterRng(seed)
    g = (np.arange(size) + 0.5) / size
    X, Y = np.meshgrid(g, g, indexing="xy")
    out = []
    for t in range(n):
        c0, c1 = rng.uniform(3, 0.05, 0.95), rng.uniform(3, 0.05, 0.95)
        period = int(rng.uniform(1, 4, 33)[0])
        mix = rng.uniform(1, 0.2, 0.8)[0]
        checker = ((np.floor(X * period) + np.floor(Y * period)) % 2).astype(np.float64)
        noise = 0.5 + 0.5 * value_noise2(X, Y, seed * 1000 + t, octaves=3, base_freq=6.0)
        w = mix * checker + (1 - mix) * noise
        rgb = c0[None, None, :] * (1 - w[..., None]) + c1[None, None, :] * w[..., None]
        img = np.empty((size, size, 4), np.uint8)
        img[..., :3] = np.clip(np.round(rgb * 255.0), 0, 255).astype(np.uint8)
        img[..., 3] = 255
        out.append(img)
    return out


def c5_scene(n_meshes=128, subdiv=6, n_textures=64, tex_size=1024, seed=5):
    """Config-5 style scene: n_meshes displaced icospheres (as icosphere_field,
    spread over a 40-unit box) on a 256 x 256-tile heightfield terrain, with
    n_textures RGBA8 textures: the terrain (Lambert) and every other sphere
    (Disney base colour) are textured.  Returns (triangles, materials,
    textures, info)."""
    tris, mats, info = icosphere_field(n_meshes=n_meshes, subdiv=subdiv, seed=seed, box=40.0, ground_half=1.0)
    tris = tris[:-2]  # the field's ground quad is replaced by the terrain
    mats = mats.copy()
    for i in range(0, n_meshes, 2):
        mats[1 + i]["TEXTURE_BASECOLOR_ID"] = (i // 2) % n_textures
    mats[0] = make_material(LAMBERT, (0.7, 0.7, 0.7), tex=n_textures - 1)
    terrain = heightfield_terrain(tiles=256, half=150.0, height=6.0, seed=seed + 1, material_id=0,
                                  shape_id=n_meshes)
    terrain["verts"][:, :3, 2] -= 8.0  # below the spheres (whose lowest point is z = 0)
    tris = canonical(np.concatenate([tris, terrain]))
    textures = procedural_textures_rgba8(n_textures, tex_size, seed + 2)
    return tris, mats, textures, info


def sky_environment(width=2048, height=1024, sun_peak=1e4, seed=3, sun_sigma_deg=1.0):
    """Lat-long RGB float32 environment (height, width, 3) in the reference's
    mapping: row 0 = +z, column c <-> u = 1 - c/width, theta = (u - 0.5)*2*pi,
    phi = (v - 0.5)*pi, dir = (cos phi cos theta, cos phi sin theta, sin phi)
    (ImageBasedLighting.cuh:46-56).  Sky gradient over z >= 0, dim ground
    colour below, plus a Gaussian sun lobe of peak `sun_peak` at a seeded
    direction (elevation 20-60 deg)."""
    rng = CounterRng(seed)
    el = np.deg2rad(20.0 + 40.0 * rng.uniform(1)[0])
    az = 2 * np.pi * rng.uniform(1)[0]
    sun = np.array([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)])
    r = np.arange(height) + 0.5
    c = np.arange(width) + 0.5
    v = 1.0 - r / height
    u = 1.0 - c / width
    phi = (v - 0.5) * np.pi
    theta = (u - 0.5) * 2 * np.pi
    cp = np.cos(phi)[:, None]
    d = np.stack([cp * np.cos(theta)[None, :], cp * np.sin(theta)[None, :],
                  np.broadcast_to(np.sin(phi)[:, None], (height, width))], -1)
    z = d[..., 2]
    horizon = np.array([1.1, 1.05, 1.0])
    zenith = np.array([0.25, 0.45, 0.95])
    t = np.sqrt(np.clip(z, 0, 1))[..., None]
    sky = horizon * (1 - t) + zenith * t
    ground = np.array([0.18, 0.16, 0.14])
    img = np.where((z >= 0)[..., None], sky, ground)
    cosang = np.clip((d * sun).sum(-1), -1, 1)
    ang = np.arccos(cosang)
    sig = np.deg2rad(sun_sigma_deg)
    lobe = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)
    img = img + lobe[..., None] * np.array([1.0, 0.95, 0.85])
    return img.astype(np.float32), sun


# --------------------------------------------------------------------------
# Parity ray sets
# --------------------------------------------------------------------------

def parity_rays(n, lo, hi, seed=1):
    """n rays (RAY records): origins uniform in [lo, hi], directions uniform
    on the unit sphere by rejection from the unit ball.  Each ray i draws from
    its own xorshift stream seeded by SplitMix64(seed, i); only correctly
    rounded float64 operations are used, so the bytes are portable."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    idx = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        s = splitmix64(np.uint64(seed) * np.uint64(0x100000001B3) + idx)
    s[s == 0] = 1

    def draw():
        nonlocal s
        s = xorshift64(s)
        return (s >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    org = np.stack([lo[k] + (hi[k] - lo[k]) * draw() for k in range(3)], 1)
    d = np.zeros((n, 3))
    todo = np.ones(n, dtype=bool)
    while todo.any():
        cand = np.stack([2.0 * draw() - 1.0 for _ in range(3)], 1)
        l2 = (cand * cand).sum(1)
        ok = todo & (l2 > 1e-4) & (l2 <= 1.0)
        d[ok] = cand[ok] / np.sqrt(l2[ok])[:, None]
        todo &= ~ok
    rays = np.zeros(n, dtype=RAY)
    rays["dir"][:, :3] = d.astype(np.float32)
    rays["org"][:, :3] = org.astype(np.float32)
    return rays


def scene_bounds(tris):
    v = tris["verts"][:, :3, :3].reshape(-1, 3)
    return v.min(0), v.max(0)
