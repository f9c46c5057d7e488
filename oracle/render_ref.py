"""CPU restatement of the reference's frame (test infrastructure only).

Restates web/js/shaders/render.js (vsParticle / fsParticle :39-98, vsGround /
fsGround :100-130) and the camera of web/js/main.js:24-62 in NumPy f32 for
small images, to check the CUDA renderer behind xpbi_render. One sample per
pixel at the pixel centre, the nearest fragment wins (the `less` depth test
of main.js:254-262; ties keep the smaller colour word). The domain-box
lines are not restated.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def look_at(eye, tgt):
    """mat4LookAt (main.js:33-43), f64 then f32, column-major."""
    eye = np.asarray(eye, np.float64)
    z = eye - np.asarray(tgt, np.float64)
    z /= np.linalg.norm(z)
    x = np.cross([0.0, 1.0, 0.0], z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    return np.array([x[0], y[0], z[0], 0, x[1], y[1], z[1], 0, x[2], y[2], z[2], 0,
                     -x @ eye, -y @ eye, -z @ eye, 1], np.float64).astype(f32)


def perspective(fov, aspect, near, far):
    """mat4Persp (main.js:44-52)."""
    f = 1.0 / math.tan(fov / 2)
    return np.array([f / aspect, 0, 0, 0, 0, f, 0, 0, 0, 0, far / (near - far), -1,
                     0, 0, near * far / (near - far), 0], np.float64).astype(f32)


def _mv(m, v, w):
    """column-major 4x4 times (v, w) for rows of v."""
    m = m.reshape(4, 4).T.astype(f32)
    h = np.concatenate([v.astype(f32), np.full((len(v), 1), w, f32)], axis=1)
    return h @ m.T


def _pack(rgb):
    q = np.rint(np.clip(rgb, 0, 1) * f32(255)).astype(np.uint64)
    return q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (np.uint64(255) << 24)


def _smooth(e0, e1, x):
    t = np.clip((x - e0) / (e1 - e0), 0, 1).astype(f32)
    return t * t * (3 - 2 * t)


def render(pos4, vel4, mat_words, eye, target, width, height, particle_radius, ground_y,
           fov=math.pi / 4, near=0.02, far=50.0, light=(0.5, 0.9, 0.35), draw_ground=True):
    """RGBA8 (height, width, 4) of the particles pos4/vel4 (material index +
    seed in pos.w), material records mat_words (8 x 16 words)."""
    V = look_at(eye, target)
    P = perspective(fov, width / height, near, far)
    Vm = V.reshape(4, 4).T
    Pm = P.reshape(4, 4).T
    # proj * view, stored column-major like the others (mat4Mul, main.js:53-62)
    VP = (Pm.astype(np.float64) @ Vm.astype(np.float64)).astype(f32).T.reshape(16)
    bg = np.array([0.10, 0.11, 0.13], f32)
    buf = np.full((height, width), (np.uint64(np.float32(1.0).view(np.uint32)) << 32), np.uint64)
    buf |= _pack(bg)
    px = (np.arange(width, dtype=f32) + f32(0.5))
    py = (np.arange(height, dtype=f32) + f32(0.5))
    X, Y = np.meshgrid(px, py)

    def plane_point(X, Y, zv):
        xn = X / f32(width) * 2 - 1
        yn = 1 - Y / f32(height) * 2
        return xn * (-zv) / P[0], yn * (-zv) / P[5]

    eye32 = np.asarray(eye, f32)
    if draw_ground:
        def hit(X, Y):
            vx, vy = plane_point(X, Y, f32(-1))
            vz = np.full_like(vx, f32(-1))
            R = Vm[:3, :3]
            d = np.stack([R[0, 0] * vx + R[1, 0] * vy + R[2, 0] * vz,
                          R[0, 1] * vx + R[1, 1] * vy + R[2, 1] * vz,
                          R[0, 2] * vx + R[1, 2] * vy + R[2, 2] * vz], -1).astype(f32)
            t = (f32(ground_y) - eye32[1]) / d[..., 1]
            return eye32 + d * t[..., None], t
        w, t = hit(X, Y)
        wx, _ = hit(X + 1, Y)
        wy, _ = hit(X, Y + 1)
        inside = (t > 0) & (np.abs(w[..., 0] - 0.5) <= 12) & (np.abs(w[..., 2] - 0.5) <= 12)
        c = _mv(VP, w.reshape(-1, 3), 1.0).reshape(height, width, 4)
        depth = c[..., 2] / c[..., 3]
        ok = inside & (depth >= 0) & (depth < 1)
        fx = np.abs(wx[..., 0] - w[..., 0]) * 4 + np.abs(wy[..., 0] - w[..., 0]) * 4
        fz = np.abs(wx[..., 2] - w[..., 2]) * 4 + np.abs(wy[..., 2] - w[..., 2]) * 4
        gx = np.abs((w[..., 0] * 4 - 0.5) % 1 - 0.5) / np.maximum(fx, 1e-4)
        gz = np.abs((w[..., 2] * 4 - 0.5) % 1 - 0.5) / np.maximum(fz, 1e-4)
        line = 1 - np.minimum(np.minimum(gx, gz), 1)
        base = np.array([0.16, 0.17, 0.20], f32)
        lc = np.array([0.24, 0.26, 0.30], f32)
        col = base + (lc - base) * (line * 0.8)[..., None]
        dc = np.sqrt((w[..., 0] - 0.5) ** 2 + (w[..., 2] - 0.5) ** 2)
        fade = _smooth(1.2, 5.0, dc)
        col = col + (bg - col) * fade[..., None]
        frag = (depth.astype(f32).view(np.uint32).astype(np.uint64) << 32) | _pack(col)
        buf = np.where(ok, np.minimum(buf, frag), buf)

    L = _mv(V, np.asarray([light], f32) / f32(np.linalg.norm(light)), 0.0)[0, :3]
    L = L / np.linalg.norm(L)
    up = _mv(V, np.asarray([[0, 1, 0]], f32), 0.0)[0, :3]
    up = up / np.linalg.norm(up)
    vcs = _mv(V, pos4[:, :3], 1.0)[:, :3]
    r = f32(particle_radius)
    for i in range(len(pos4)):
        vc = vcs[i]
        if not vc[2] < -near:
            continue
        wpos = f32(pos4[i, 3])
        mw = mat_words[int(min(int(wpos), 7)) * 16:][:16]
        kind = float(mw[3])
        colr = mw[8:11].view(np.float32) * (f32(0.88) + f32(0.24) * (f32(wpos % 1) * f32(2.04)))
        speed = np.sqrt(np.sum(vel4[i, :3].astype(f32) ** 2))
        qx, qy = plane_point(X, Y, vc[2])
        u, v = (qx - vc[0]) / r, (qy - vc[1]) / r
        r2 = u * u + v * v
        m = r2 <= 1
        if not m.any():
            continue
        nz = np.sqrt(np.maximum(1 - r2, 0))
        n = np.stack([u, v, nz], -1)
        vp = vc + n * r
        cp = _mv(P, vp.reshape(-1, 3), 1.0).reshape(height, width, 4)
        depth = cp[..., 2] / cp[..., 3]
        m &= (depth >= 0) & (depth < 1)
        diff = np.maximum(n @ L, 0)
        hemi = 0.5 + 0.5 * (n @ up)
        col = colr * (0.35 + 0.55 * diff + 0.35 * hemi * 0.5)[..., None]
        if kind > 5.5:
            f1 = 1 - nz
            col = col + (np.array([0.75, 0.9, 1.0], f32) - col) * (f1 * f1 * 0.6)[..., None]
            col = col + (np.array([0.85, 0.95, 1.0], f32) - col) * min(max(speed * 0.25, 0), 0.45)
        Vd = -vp / np.linalg.norm(vp, axis=-1, keepdims=True)
        H = L + Vd
        H = H / np.linalg.norm(H, axis=-1, keepdims=True)
        spec = np.clip(np.sum(n * H, -1), 0, 1) ** 48 * (0.6 if kind > 5.5 else 0.15)
        col = col + spec[..., None]
        frag = (depth.astype(f32).view(np.uint32).astype(np.uint64) << 32) | _pack(col)
        buf = np.where(m, np.minimum(buf, frag), buf)
    out = (buf & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    return out.view(np.uint8).reshape(height, width, 4)
