"""Oracle: the rasteriser that consumes the deformed Gaussians.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The viewer draws the deformed field with the external CudaRasterizer's
``forward`` (call sites GaussianView.cpp:1066-1127).  Its source is not in the
reference tree, so this is **parity unpinned**.  What follows restates, in
numpy, the published 3D Gaussian splatting method (Kerbl et al., SIGGRAPH
2023), with EWA splatting (Zwicker et al., 2002) for the projection.  The
window and the GL interop are replaced by an image array.

Matrices are row-major numpy 4x4: ``view`` maps world to camera, ``proj``
maps world to clip space.  Per Gaussian:
- it is culled when its camera-space depth is at most 0.2;
- its 3D covariance is R diag(m s)^2 R^T, for scale modifier m;
- its 2D covariance is J W Sigma W^T J^T plus 0.3 on the diagonal, where W is
  the view rotation and J the perspective Jacobian at the camera-space mean.
  Before J is formed, x/z and y/z are clamped to 1.3 tan(fov/2);
- its radius is ceil(3 sqrt(largest eigenvalue)), with the eigenvalue's
  discriminant floored at 0.1;
- its colour is the SH value in direction (mu - campos)/|mu - campos|, plus
  0.5, clamped at 0;
- it covers the 16x16 tiles its radius square touches.

Per pixel, the Gaussians of the pixel's tile are composited front to back by
camera depth, ties by index:
- alpha = min(0.99, o exp(power)), with power the conic form at the pixel
  offset; a term with power > 0 or alpha < 1/255 is skipped;
- compositing stops before a term would take the transmittance T below 1e-4;
- the pixel is sum of c alpha T, plus T times the background.

The SH basis is the real basis with the Condon-Shortley phase (sign
(-1)^|m|), in the interleaved order [coefficient][rgb] of the viewer's
``SHs<3>``.  Its constant term is helper.hpp:60's SH0.  Flipping the sign of
its odd coefficients gives the phase-free basis.  That flip is the one the
viewer's SH rotation applies around its band rotation (GaussianView.cpp:3138-3154),
so rotating coefficients with ``oracle.skin.rotate_sh`` rotates the colour
this basis gives.
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special

F64 = np.float64
TILE = 16


def sh_basis(dirs, degree=3):
    """[M,(degree+1)^2] basis values at unit directions [M,3]."""
    d = np.asarray(dirs, F64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    theta = np.arccos(np.clip(d[:, 2], -1.0, 1.0))      # polar angle from +z
    phi = np.arctan2(d[:, 1], d[:, 0])
    out = np.empty((d.shape[0], (degree + 1) ** 2))
    for l in range(degree + 1):
        for m in range(-l, l + 1):
            Y = special.sph_harm_y(l, abs(m), theta, phi)   # complex, with the phase (-1)^m
            if m > 0:
                real = math.sqrt(2) * (-1) ** m * Y.real
            elif m < 0:
                real = math.sqrt(2) * (-1) ** m * Y.imag
            else:
                real = Y.real
            out[:, l * l + l + m] = (-1) ** abs(m) * real
    return out


def sh_color(shs, dirs, degree=3):
    """RGB [M,3] of interleaved SH [M,48] in directions [M,3] (no offset)."""
    B = sh_basis(dirs, degree)
    c = np.asarray(shs, F64).reshape(-1, 16, 3)[:, :B.shape[1]]
    return np.einsum("mk,mkc->mc", B, c)


def _quat_to_matrix(q):
    q = np.asarray(q, F64)
    q = q / np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def preprocess(pos, shs, opacity, scale, rot, view, proj, campos, tan_fovx, tan_fovy, width, height,
               sh_degree=3, scale_modifier=1.0):
    """Per Gaussian: visible flag, pixel mean [N,2], conic [N,3] (a, b, c of
    the inverse 2D covariance), radius, depth, colour [N,3] and tile rect
    (x0, y0, x1, y1), x1/y1 exclusive."""
    p = np.asarray(pos, F64)
    N = p.shape[0]
    V = np.asarray(view, F64)
    P = np.asarray(proj, F64)
    ph = np.concatenate([p, np.ones((N, 1))], axis=1)
    pv = ph @ V.T
    depth = pv[:, 2]
    visible = depth > 0.2
    clip = ph @ P.T
    ndc = clip[:, :3] / (clip[:, 3:4] + 1e-7)
    Rg = _quat_to_matrix(rot)
    s = np.asarray(scale, F64) * scale_modifier
    Sig = np.einsum("nij,nj,nkj->nik", Rg, s * s, Rg)
    fx = width / (2.0 * tan_fovx)
    fy = height / (2.0 * tan_fovy)
    tz = np.where(visible, depth, 1.0)
    tx = np.clip(pv[:, 0] / tz, -1.3 * tan_fovx, 1.3 * tan_fovx) * tz
    ty = np.clip(pv[:, 1] / tz, -1.3 * tan_fovy, 1.3 * tan_fovy) * tz
    J = np.zeros((N, 2, 3))
    J[:, 0, 0] = fx / tz
    J[:, 0, 2] = -fx * tx / (tz * tz)
    J[:, 1, 1] = fy / tz
    J[:, 1, 2] = -fy * ty / (tz * tz)
    T = J @ V[:3, :3]
    C2 = np.einsum("nij,njk,nlk->nil", T, Sig, T)
    a = C2[:, 0, 0] + 0.3
    b = C2[:, 0, 1]
    c = C2[:, 1, 1] + 0.3
    det = a * c - b * b
    visible &= det != 0
    det = np.where(det != 0, det, 1.0)
    conic = np.stack([c / det, -b / det, a / det], axis=1)
    mid = 0.5 * (a + c)
    root = np.sqrt(np.maximum(0.1, mid * mid - det))
    radius = np.ceil(3.0 * np.sqrt(np.maximum(mid + root, mid - root)))
    px = ((ndc[:, 0] + 1.0) * width - 1.0) * 0.5
    py = ((ndc[:, 1] + 1.0) * height - 1.0) * 0.5
    gx = (width + TILE - 1) // TILE
    gy = (height + TILE - 1) // TILE
    x0 = np.clip(((px - radius) / TILE).astype(np.int64), 0, gx)
    y0 = np.clip(((py - radius) / TILE).astype(np.int64), 0, gy)
    x1 = np.clip(((px + radius + TILE - 1) / TILE).astype(np.int64), 0, gx)
    y1 = np.clip(((py + radius + TILE - 1) / TILE).astype(np.int64), 0, gy)
    visible &= (x1 - x0) * (y1 - y0) > 0
    dirs = p - np.asarray(campos, F64)[None]
    col = np.maximum(sh_color(shs, dirs, sh_degree) + 0.5, 0.0)
    return {"visible": visible, "xy": np.stack([px, py], 1), "conic": conic, "radius": radius,
            "depth": depth, "color": col, "opacity": np.asarray(opacity, F64),
            "rect": np.stack([x0, y0, x1, y1], 1)}


def render(pos, shs, opacity, scale, rot, view, proj, campos, tan_fovx, tan_fovy, width, height,
           background=(0.0, 0.0, 0.0), sh_degree=3, scale_modifier=1.0):
    """(image [3,H,W], final transmittance [H,W], contributors [H,W])."""
    g = preprocess(pos, shs, opacity, scale, rot, view, proj, campos, tan_fovx, tan_fovy, width, height,
                   sh_degree, scale_modifier)
    N = g["depth"].shape[0]
    order = np.lexsort((np.arange(N), g["depth"]))
    img = np.zeros((3, height, width))
    Tf = np.ones((height, width))
    ncon = np.zeros((height, width), np.int64)
    bg = np.asarray(background, F64)
    for ty in range((height + TILE - 1) // TILE):
        for tx in range((width + TILE - 1) // TILE):
            ids = [i for i in order if g["visible"][i] and g["rect"][i, 0] <= tx < g["rect"][i, 2]
                   and g["rect"][i, 1] <= ty < g["rect"][i, 3]]
            for y in range(ty * TILE, min(height, ty * TILE + TILE)):
                for x in range(tx * TILE, min(width, tx * TILE + TILE)):
                    T = 1.0
                    C = np.zeros(3)
                    n = 0
                    for i in ids:
                        dx = g["xy"][i, 0] - x
                        dy = g["xy"][i, 1] - y
                        ca, cb, cc = g["conic"][i]
                        power = -0.5 * (ca * dx * dx + cc * dy * dy) - cb * dx * dy
                        if power > 0.0:
                            continue
                        alpha = min(0.99, g["opacity"][i] * math.exp(power))
                        if alpha < 1.0 / 255.0:
                            continue
                        t_next = T * (1.0 - alpha)
                        if t_next < 1e-4:
                            break
                        C += g["color"][i] * alpha * T
                        T = t_next
                        n += 1
                    img[:, y, x] = C + T * bg
                    Tf[y, x] = T
                    ncon[y, x] = n
    return img, Tf, ncon
