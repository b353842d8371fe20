"""Test infrastructure: a numpy restatement of the reference's display
variables and of the arithmetic of its heat-map, volume and LIC shaders, the
checker for the library's headless views.  Nothing here is used by the
library.

  display variables   hydro/eqn/euler.lua:240-260, hydro/eqn/eqn.lua:913-915,
                      hydro/eqn/euler.cl:1-131 (the expressions, in double)
  display buffer      hydro/solver/solverbase.lua:1950-2065 (ghost clamp,
                      zeroBorder)
  range / mean / dev  hydro/solver/solverbase.lua:2871-2994
  palette mapping     hydro/draw/draw.glsl:43-85, hydro/draw/palette.lua,
                      hydro/app.lua:1229-1241
  heat map            hydro/draw/2d_heatmap.glsl:28-59
  volume              hydro/draw/volumetric.glsl:36-110
  LIC                 hydro/draw/vector_lic.glsl:36-107

Pixel colours are not pinned to the reference: they depend on the graphics
driver's filtering precision and on the gradient texture class of lua-gl
(GLGradientTex2D), neither of which is part of the reference; this module
restates the documented behaviour (linear filtering, repeat wrap, colours
interpolated linearly along the texture) in float32.
"""
import numpy as np

DISPLAY_VARS = ["rho", "m x", "m y", "m z", "m mag", "ETotal", "ePot", "v x", "v y", "v z", "v mag", "P",
                "eInt", "eKin", "eTotal", "EInt", "EKin", "EPot", "S", "H", "h", "HTotal", "hTotal",
                "speed of sound", "Mach number", "temperature"]
AIR_CV = 717.1   # hydro/materials.lua:61
GRAD_W = 1024
G = 2


def display_values(U, var, gamma, rhoMin=1e-7, PMin=1e-7):
    """The display variable of each cell of U (cells, 6), in double."""
    U = np.asarray(U, dtype=np.float64)
    rho, mx, my, mz, E, ePot = (U[..., k] for k in range(6))
    with np.errstate(all="ignore"):
        inv = 1. / rho
        vx, vy, vz = mx * inv, my * inv, mz * inv
        EKinC = np.where(rho < rhoMin, 0., .5 * (mx * mx + my * my + mz * mz) / rho)
        P = np.where(rho < rhoMin, 0., (gamma - 1.) * (E - EKinC))
        Cs = np.where(P <= PMin, 0., np.where(rho < rhoMin, np.inf, np.sqrt(gamma * P / rho)))
        vsq = vx * vx + vy * vy + vz * vz
        name = DISPLAY_VARS[var] if not isinstance(var, str) else var
        return {
            "rho": rho, "m x": mx, "m y": my, "m z": mz, "m mag": np.sqrt(mx * mx + my * my + mz * mz),
            "ETotal": E, "ePot": ePot, "v x": vx, "v y": vy, "v z": vz, "v mag": np.sqrt(vsq), "P": P,
            "eInt": (P / (gamma - 1.)) / rho, "eKin": .5 * vsq, "eTotal": E / rho, "EInt": P / (gamma - 1.),
            "EKin": rho * (.5 * vsq), "EPot": rho * ePot, "S": P / np.power(rho, gamma),
            "H": P * (gamma / (gamma - 1.)), "h": P * (gamma / (gamma - 1.)) / rho, "HTotal": P + E,
            "hTotal": (P + E) / rho, "speed of sound": Cs, "Mach number": np.sqrt(vsq) / Cs,
            "temperature": ((E - .5 * (mx * mx + my * my + mz * mz) / rho) / rho - ePot) / AIR_CV,
        }[name]


def display_buffer(U_grid, var, gamma, zero_border=False, **eos):
    """calcDisplayVarToBuffer over the ghost-inclusive grid.  U_grid: interior
    cells shaped (nz, ny, nx, 6) (unused axes of size 1); returns the grid
    with 2 ghost layers on each active axis."""
    nz, ny, nx, _ = U_grid.shape
    dim = 3 if nz > 1 else (2 if ny > 1 else 1)
    v = display_values(U_grid, var, gamma, **eos)
    pads = [(G, G) if a < dim else (0, 0) for a in (2, 1, 0)]   # z, y, x
    out = np.pad(v, pads, mode="edge")
    if zero_border:
        mask = np.zeros(out.shape, dtype=bool)
        sl = tuple(slice(G, -G) if p[0] else slice(None) for p in pads)
        mask[sl] = True
        out = np.where(mask, out, 0.)
    return out


def display_range(U_grid, var, gamma, **eos):
    v = display_values(U_grid, var, gamma, **eos).ravel()
    m = v.sum() / v.size
    return v.min(), v.max(), m, np.sqrt(((v - m) ** 2).sum() / v.size)


PALETTES = {
    0: [(0, 0, 1, .8), (0, 1, 1, .8), (0, 1, 0, .8), (1, 1, 0, .8), (1, .5, 0, .8), (1, 0, 0, .8), (1, 1, 1, .8)],
    1: [(1, 1, 1, 1) if i % 2 == 1 else (0, 0, 0, 0) for i in range(1, 33)],
    2: [(0, 0, 0, .8), (.5, .5, 1, .8), (1, 1, 1, .8)],
    3: [tuple(int(h[k:k + 2], 16) / 255. for k in (0, 2, 4)) + (1.,) for h in ("3c4ec2", "dddddd", "b40426")],
}


def gradient_texture(palette=0):
    """(GRAD_W, 4) float32: texel i at position i/(W-1) along the colour list."""
    cols = np.array(PALETTES[palette], dtype=np.float64)
    n = len(cols)
    f = np.arange(GRAD_W) / (GRAD_W - 1) * (n - 1)
    lo = np.clip(np.floor(f).astype(int), 0, n - 2)
    t = (f - lo)[:, None]
    return ((1 - t) * cols[lo] + t * cols[lo + 1]).astype(np.float32)


def _wrap(i, n):
    return np.mod(i, n)


def sample_linear(tex, u, v=None, w=None):
    """GL_LINEAR + GL_REPEAT sampling of tex (d, h, w, comps) at normalised
    coordinates (float32 arithmetic)."""
    f32 = np.float32
    D, H, W, C = tex.shape
    u = np.asarray(u, dtype=f32)
    v = np.full_like(u, f32(.5)) if v is None else np.asarray(v, dtype=f32)
    w = np.full_like(u, f32(.5)) if w is None else np.asarray(w, dtype=f32)
    x, y, z = u * f32(W) - f32(.5), v * f32(H) - f32(.5), w * f32(D) - f32(.5)
    fx, fy, fz = np.floor(x), np.floor(y), np.floor(z)
    ax, ay, az = x - fx, y - fy, z - fz
    x0, y0, z0 = fx.astype(np.int64), fy.astype(np.int64), fz.astype(np.int64)
    acc = np.zeros(u.shape + (C,), dtype=f32)
    for dz in range(2 if D > 1 else 1):
        for dy in range(2 if H > 1 else 1):
            for dx in range(2):
                wgt = (ax if dx else f32(1) - ax)
                if H > 1:
                    wgt = wgt * (ay if dy else f32(1) - ay)
                if D > 1:
                    wgt = wgt * (az if dz else f32(1) - az)
                t = tex[_wrap(z0 + dz, D), _wrap(y0 + dy, H), _wrap(x0 + dx, W)]
                acc = acc + wgt[..., None] * t
    return acc


def gradient_frac(value, vmin, vmax, use_log=False):
    f32 = np.float32
    value = np.asarray(value, dtype=f32)
    vmin, vmax = f32(vmin), f32(vmax)
    if use_log:
        lg = lambda x: np.log(np.abs(x)) * f32(1. / np.log(10.))
        lo, hi = lg(vmin), lg(vmax)
        if (vmin < 0) != (vmax < 0):
            lo = f32(0)
        elif vmin < 0:
            lo, hi = hi, lo
        return (lg(value) - lo) / (hi - lo)
    return (value - vmin) / (vmax - vmin)


def gradient_color(grad, frac):
    tc = (np.asarray(frac, dtype=np.float32) * np.float32(GRAD_W - 1) + np.float32(.5)) * np.float32(1. / GRAD_W)
    return sample_linear(grad.reshape(1, 1, GRAD_W, 4), tc)


def to_rgba8(c):
    c = np.nan_to_num(np.asarray(c, dtype=np.float32), nan=0.)
    return np.rint(np.clip(c, 0, 1) * np.float32(255)).astype(np.uint8)


def _quat_rotate(q, x, y, z):
    qx, qy, qz, qw = (np.float32(a) for a in q)
    tx = qy * z - qz * y + qw * x
    ty = qz * x - qx * z + qw * y
    tz = qx * y - qy * x + qw * z
    return (x + np.float32(2) * (qy * tz - qz * ty), y + np.float32(2) * (qz * tx - qx * tz),
            z + np.float32(2) * (qx * ty - qy * tx))


class _Frame:
    def __init__(self, desc_dim, n, mins, maxs):
        f32 = np.float32
        self.dim = desc_dim
        self.mins = [f32(m) for m in mins]
        self.maxs = [f32(m) for m in maxs]
        self.grid = [f32(n[k] + 4) if k < desc_dim else f32(5) for k in range(3)]
        self.size = [f32(n[k]) if k < desc_dim else f32(1) for k in range(3)]

    def chart_to_tex(self, x, k):
        return ((x - self.mins[k]) / (self.maxs[k] - self.mins[k]) * self.size[k] + np.float32(2)) / self.grid[k]

    def tex_to_no_ghost(self, t, k):
        return (t * self.size[k] + np.float32(2)) / self.grid[k]


def _pixels(width, height, bbox):
    f32 = np.float32
    py, px = np.mgrid[0:height, 0:width].astype(f32)
    sx, sy = (px + f32(.5)) / f32(width), (py + f32(.5)) / f32(height)
    b = [f32(v) for v in bbox]
    return b[0] + (b[2] - b[0]) * sx, b[1] + (b[3] - b[1]) * sy


def heatmap(tex, dim, n, mins, maxs, width, height, bbox, vmin, vmax, palette=0, use_log=False,
            q=(0, 0, 0, 1), fixed_z=0.):
    """tex: the float32 display texture (d, h, w); returns (height, width, 4) uint8."""
    fr = _Frame(dim, n, mins, maxs)
    x, y = _pixels(width, height, bbox)
    z = np.full_like(x, np.float32(fixed_z))
    x, y, z = _quat_rotate(q, x, y, z)
    tx, ty, tz = fr.chart_to_tex(x, 0), fr.chart_to_tex(y, 1), fr.chart_to_tex(z, 2)
    out = (tx < 0) | (tx > 1)
    if dim > 1:
        out |= (ty < 0) | (ty > 1)
    if dim > 2:
        out |= (tz < 0) | (tz > 1)
    val = sample_linear(tex[..., None], tx, ty, tz)[..., 0]
    c = gradient_color(gradient_texture(palette), gradient_frac(val, vmin, vmax, use_log))
    img = to_rgba8(c)
    img[out] = 0
    return img


def _smoothstep(e0, e1, x):
    f32 = np.float32
    t = np.clip((x - f32(e0)) / (f32(e1) - f32(e0)), f32(0), f32(1))
    return t * t * (f32(3) - f32(2) * t)


def lic(vel, noise, dim, n, mins, maxs, width, height, bbox, vmin, vmax, palette=0, iters=10,
        q=(0, 0, 0, 1), fixed_z=0.):
    """vel: float32 (d, h, w, 4) velocity texture; noise: float32 (N, N)."""
    f32 = np.float32
    fr = _Frame(dim, n, mins, maxs)
    N = noise.shape[0]
    ntex = noise.reshape(1, N, N, 1)
    x, y = _pixels(width, height, bbox)
    z = np.full_like(x, f32(fixed_z))
    x, y, z = _quat_rotate(q, x, y, z)
    tx, ty, tz = fr.chart_to_tex(x, 0), fr.chart_to_tex(y, 1), fr.chart_to_tex(z, 2)
    outside = (tx < 0) | (tx > 1) | (ty < 0) | (ty > 1)
    if dim > 2:
        outside |= (tz < 0) | (tz > 1)

    def ng(a, b, c):
        return (fr.tex_to_no_ghost(fr.chart_to_tex(a, 0), 0), fr.tex_to_no_ghost(fr.chart_to_tex(b, 1), 1),
                fr.tex_to_no_ghost(fr.chart_to_tex(c, 2), 2))

    g0 = ng(x, y, z)
    licv = sample_linear(ntex, g0[0], g0[1])[..., 0]
    total = np.ones_like(licv)
    ds = f32(1) / f32(N)
    for d in (-1, 1):
        px, py_, pz = x.copy(), y.copy(), z.copy()
        last = np.zeros(x.shape + (3,), dtype=f32)
        alive = np.ones(x.shape, dtype=bool)
        for it in range(iters):
            q0 = ng(px, py_, pz)
            u = sample_linear(vel, q0[0], q0[1], q0[2])[..., :3]
            if it > 0:
                alive &= ~((u * last).sum(-1) < 0)
            m = np.sqrt((u * u).sum(-1))
            alive &= ~(m == 0)
            with np.errstate(all="ignore"):
                s = np.where(alive, ds * f32(d) / m, f32(0))
            px = np.where(alive, px + u[..., 0] * s, px)
            py_ = np.where(alive, py_ + u[..., 1] * s, py_)
            pz = np.where(alive, pz + u[..., 2] * s, pz)
            f = f32(it + 1) / f32(iters + 1)
            wgt = _smoothstep(1., 0., f)
            qn = ng(px, py_, pz)
            licv = np.where(alive, licv + sample_linear(ntex, qn[0], qn[1])[..., 0] * wgt, licv)
            total = np.where(alive, total + wgt, total)
            last = np.where(alive[..., None], u, last)
    licv = _smoothstep(.2, .8, licv / total)
    u0 = sample_linear(vel, g0[0], g0[1], g0[2])[..., :3]
    mag = np.clip(np.sqrt((u0 * u0).sum(-1)), f32(vmin), f32(vmax))
    c = gradient_color(gradient_texture(palette), gradient_frac(mag, vmin, vmax))
    c[..., :3] *= licv[..., None]
    img = to_rgba8(c)
    img[outside] = 0
    return img


def splitmix_uniforms(seed, n):
    """The first n uniforms in [0, 1) of SplitMix64(seed) as float32."""
    M = (1 << 64) - 1
    out = np.empty(n, dtype=np.float64)
    for k in range(n):
        z = (seed + (k + 1) * 0x9E3779B97F4A7C15) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z = z ^ (z >> 31)
        out[k] = (z >> 11) * (1.0 / 9007199254740992.0)
    return out.astype(np.float32)


def camera(eye, mins, maxs, fov_y, width, height):
    """Rays of the volume view: a pinhole at `eye` looking at the domain's
    centre, y up (z up when looking along y).  Returns (fwd, right, up,
    tan(fov/2)) in float32."""
    c = (np.asarray(mins, dtype=np.float64) + np.asarray(maxs, dtype=np.float64)) * .5
    f = c - np.asarray(eye, dtype=np.float64)
    f /= np.sqrt((f * f).sum())
    up = np.array([0., 0., 1.]) if abs(f[1]) > .999 else np.array([0., 1., 0.])
    r = np.cross(f, up)
    r /= np.sqrt((r * r).sum())
    u = np.cross(r, f)
    return f.astype(np.float32), r.astype(np.float32), u.astype(np.float32), np.float32(np.tan(fov_y * np.pi / 360.))


def volume(tex, n, mins, maxs, width, height, vmin, vmax, eye, fov_y=45., palette=0, alpha=.15, alpha_gamma=1.,
           max_iter=100, use_isobars=False, num_isobars=10., use_lighting=False, use_log=False):
    """volumetric.glsl's march from each pixel ray's entry into the domain box."""
    f32 = np.float32
    fr = _Frame(3, n, mins, maxs)
    grad = gradient_texture(palette)
    fwd, rt, up, th = camera(eye, mins, maxs, fov_y, width, height)
    py, px = np.mgrid[0:height, 0:width].astype(f32)
    sx = ((px + f32(.5)) / f32(width) * f32(2) - f32(1)) * th * (f32(width) / f32(height))
    sy = ((py + f32(.5)) / f32(height) * f32(2) - f32(1)) * th
    d = [fwd[k] + sx * rt[k] + sy * up[k] for k in range(3)]
    e = [f32(v) for v in eye]
    mn, mx = [f32(v) for v in mins], [f32(v) for v in maxs]
    t0 = np.zeros_like(sx)
    t1 = np.full_like(sx, np.inf)
    with np.errstate(all="ignore"):
        for a in range(3):
            zero = d[a] == 0
            ta, tb = (mn[a] - e[a]) / d[a], (mx[a] - e[a]) / d[a]
            lo, hi = np.minimum(ta, tb), np.maximum(ta, tb)
            t0 = np.where(zero, np.where((e[a] < mn[a]) | (e[a] > mx[a]), np.inf, t0), np.maximum(t0, lo))
            t1 = np.where(zero, t1, np.minimum(t1, hi))
    hit = (t0 <= t1) & (t0 < np.inf)
    t0 = np.where(hit, t0, f32(0))
    start = [e[k] + t0 * d[k] for k in range(3)]
    p = [(start[k] - mn[k]) / (mx[k] - mn[k]) for k in range(3)]

    def voxel(q):
        tq = [q[k] * (fr.size[k] / fr.grid[k]) + f32(2) / fr.grid[k] for k in range(3)]
        with np.errstate(all="ignore"):
            return sample_linear(tex[..., None], tq[0], tq[1], tq[2])[..., 0]

    rgb = np.zeros(sx.shape + (3,), dtype=f32)
    ra = np.ones_like(sx)
    c = gradient_color(grad, gradient_frac(voxel(p), vmin, vmax, use_log))
    a = f32(alpha) * np.minimum(f32(1), np.sqrt((c[..., :3] ** 2).sum(-1)))
    rgb += (ra * a)[..., None] * c[..., :3]
    ra = ra * (f32(1) - a)
    dd = [start[k] - e[k] for k in range(3)]
    with np.errstate(all="ignore"):
        inv = f32(1) / (np.sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) * f32(max_iter))
        # a ray that misses the box has no step (0/0): it stays where it is, at
        # finite coordinates, and is masked out of the composite below
        step = [np.where(hit, dd[k] * inv, f32(0)) for k in range(3)]
    alive = hit.copy()
    for i in range(2, max_iter + 1):
        p = [p[k] + step[k] for k in range(3)]
        alive &= ~((p[0] < 0) | (p[1] < 0) | (p[2] < 0) | (p[0] > 1) | (p[1] > 1) | (p[2] > 1))
        if not alive.any():
            break
        frac = gradient_frac(voxel(p), vmin, vmax, use_log)
        c = gradient_color(grad, frac)
        if use_isobars:
            ff = frac * f32(num_isobars) + f32(.5)
            ffrac = ff - np.floor(ff)
            a = _smoothstep(0., .1 / 3., ffrac) - _smoothstep(2. / 3. * .1, .1, ffrac)
        else:
            a = np.full_like(sx, f32(alpha) ** f32(alpha_gamma))
        if use_lighting:
            h = f32(1. / 32.)
            gx = voxel([p[0] + h, p[1], p[2]]) - voxel([p[0] - h, p[1], p[2]])
            gy = voxel([p[0], p[1] + h, p[2]]) - voxel([p[0], p[1] - h, p[2]])
            gz = voxel([p[0], p[1], p[2] + h]) - voxel([p[0], p[1], p[2] - h])
            with np.errstate(all="ignore"):
                g = np.abs(gz / np.sqrt(gx * gx + gy * gy + gz * gz))
            # GLSL max(x, y) = x < y ? y : x: a flat region's NaN gives the ambient term
            lum = np.where(f32(.3) < g, g, f32(.3))
            c = c * lum[..., None]
        a = np.where(alive, a, f32(0))
        rgb += (ra * a)[..., None] * c[..., :3]
        ra = ra * (f32(1) - a)
    img = to_rgba8(np.concatenate([rgb, (f32(1) - ra)[..., None]], axis=-1))
    img[~hit] = 0
    return img


def slices(tex, n, width, height, vmin, vmax, axis=2, num_slices=255, palette=0, alpha=.15, alpha_gamma=1.,
           use_isobars=True, num_isobars=20., use_lighting=False, q=(0, 0, 0, 1), use_log=False):
    """3d_slice.lua's slice stack as an orthographic view along `axis` (0..2
    towards +axis, 3..5 towards -axis), blended back to front with
    (SRC_ALPHA, ONE_MINUS_SRC_ALPHA); per slice 3d_slice.glsl's fragment with
    the projection factor taken as 1."""
    f32 = np.float32
    fr = _Frame(3, n, [0, 0, 0], [1, 1, 1])
    grad = gradient_texture(palette)
    ax = axis % 3
    plus = axis < 3
    a1, a2 = (1 if ax == 0 else 0), (1 if ax == 2 else 2)
    py, px = np.mgrid[0:height, 0:width].astype(f32)
    u, v = (px + f32(.5)) / f32(width), (py + f32(.5)) / f32(height)
    rgb = np.zeros(u.shape + (3,), dtype=f32)
    acc = np.zeros_like(u)

    def voxel(q3):
        with np.errstate(all="ignore"):
            return sample_linear(tex[..., None], q3[0], q3[1], q3[2])[..., 0]

    for s in range(num_slices + 1):
        j = num_slices - s if plus else s
        f = f32(j) / f32(num_slices)
        c = [None, None, None]
        c[ax] = np.full_like(u, f)
        c[a1], c[a2] = u, v
        tx, ty, tz = _quat_rotate(q, c[0], c[1], c[2])
        inside = ~((tx < 0) | (tx > 1) | (ty < 0) | (ty > 1) | (tz < 0) | (tz > 1))
        ng = [fr.tex_to_no_ghost(t, k) for k, t in enumerate((tx, ty, tz))]
        frac = gradient_frac(voxel(ng), vmin, vmax, use_log)
        col = gradient_color(grad, frac)
        if use_isobars:
            ff = frac * f32(num_isobars) + f32(.5)
            ffrac = ff - np.floor(ff)
            a = _smoothstep(0., .1 / 3., ffrac) - _smoothstep(2. / 3. * .1, .1, ffrac)
        else:
            a = np.full_like(u, f32(alpha) ** f32(alpha_gamma))
        if use_lighting:
            h = f32(1. / 32.)
            gx = voxel([ng[0] + h, ng[1], ng[2]]) - voxel([ng[0] - h, ng[1], ng[2]])
            gy = voxel([ng[0], ng[1] + h, ng[2]]) - voxel([ng[0], ng[1] - h, ng[2]])
            gz = voxel([ng[0], ng[1], ng[2] + h]) - voxel([ng[0], ng[1], ng[2] - h])
            with np.errstate(all="ignore"):
                g = np.abs(gz / np.sqrt(gx * gx + gy * gy + gz * gz))
            col = col * np.where(f32(.3) < g, g, f32(.3))[..., None]
        sa = np.where(inside, a * f32(alpha), f32(0))
        rgb = np.where(inside[..., None], col[..., :3] * sa[..., None] + rgb * (f32(1) - sa)[..., None], rgb)
        acc = np.where(inside, sa * sa + acc * (f32(1) - sa), acc)
    return to_rgba8(np.concatenate([rgb, acc[..., None]], axis=-1))
