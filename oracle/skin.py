"""Oracle: Gaussian refit from six deformed endpoints, SH rotation, sample skinning.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restated from:

* ``end_points``        -- GaussianView.cpp:4643-4668 (GetEndPoints)
* ``refit_gaussians``   -- GaussianView.cpp:3081-3166 (UpdateAsSixPointsWithdrawBad)
                           with helper.cpp:429-440 (getOthogonalMatrixWithK)
* ``quat_from_matrix``  -- the conversion Eigen performs for
                           ``Quaternionf(Matrix3f)`` at GaussianView.cpp:3119;
                           restated from Shoemake's published method
* ``sh_rotation_matrices`` / ``rotate_sh`` -- helper.cpp:938-1075 and
                           cudakdtree.cu:11-199; restated from the
                           Ivanic-Ruedenberg recurrence for real SH rotation
                           (J. Phys. Chem. 100 (1996) 6342, erratum 102 (1998)
                           9099) and pinned to the reference's unrolled
                           formulas by ``tests/golden/sh_rotation.json``
* ``node_quaternions``  -- GaussianView.cpp:3169-3186 with helper.cpp:506-517
                           (FastgetOthogonalMatrix) and helper.cpp:816-820
* ``slerp_blend``       -- cudakdtree.cu:113-148, 201-222 (Q_SlerpCUDA, RotateSHs)
* ``static masks``      -- GaussianView.cpp:2038-2070 (CheckStaticSamples)

Per-item 3x3, quaternion and SH arithmetic is evaluated in float64 and rounded
to float32 where the reference stores float32 (positions, endpoints,
quaternions, scales, SH).  Branch decisions that the reference takes on float32
values (the slerp cosine threshold, the polar-iteration stop) are taken on the
same float32 values here.
"""
from __future__ import annotations

import numpy as np

from . import ed as _ed

F32 = np.float32
F64 = np.float64

END_COEFF = F32(2.0)      # GaussianView.hpp:116
AXIS_PADDING = F32(1e-3)  # GaussianView.hpp:117


# ------------------------------------------------------------ quaternions --

def quat_to_matrix(q):
    """Unit quaternion (w,x,y,z) [...,4] -> rotation matrix [...,3,3] (row-major)."""
    q = np.asarray(q, F64)
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3), F64)
    R[..., 0, 0] = 1 - 2 * (y * y + z * z)
    R[..., 0, 1] = 2 * (x * y - w * z)
    R[..., 0, 2] = 2 * (x * z + w * y)
    R[..., 1, 0] = 2 * (x * y + w * z)
    R[..., 1, 1] = 1 - 2 * (x * x + z * z)
    R[..., 1, 2] = 2 * (y * z - w * x)
    R[..., 2, 0] = 2 * (x * z - w * y)
    R[..., 2, 1] = 2 * (y * z + w * x)
    R[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def quat_normalize(q):
    q = np.asarray(q, F64)
    return q / np.linalg.norm(q, axis=-1, keepdims=True)


def quat_mul(a, b):
    aw, ax, ay, az = (a[..., i] for i in range(4))
    bw, bx, by, bz = (b[..., i] for i in range(4))
    return np.stack([aw * bw - ax * bx - ay * by - az * bz,
                     aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw], axis=-1)


def quat_inverse(q):
    q = np.asarray(q, F64)
    c = q * np.array([1.0, -1.0, -1.0, -1.0])
    return c / (q * q).sum(-1, keepdims=True)


def quat_from_matrix(M):
    """Shoemake's trace/largest-diagonal method, (w,x,y,z) [...,4] (not normalised)."""
    M = np.asarray(M, F64)
    shp = M.shape[:-2]
    M = M.reshape(-1, 3, 3)
    q = np.empty((M.shape[0], 4), F64)
    tr = M[:, 0, 0] + M[:, 1, 1] + M[:, 2, 2]
    pos = tr > 0
    if pos.any():
        m = M[pos]
        t = np.sqrt(tr[pos] + 1.0)
        s = 0.5 / t
        q[pos, 0] = 0.5 * t
        q[pos, 1] = (m[:, 2, 1] - m[:, 1, 2]) * s
        q[pos, 2] = (m[:, 0, 2] - m[:, 2, 0]) * s
        q[pos, 3] = (m[:, 1, 0] - m[:, 0, 1]) * s
    neg = np.flatnonzero(~pos)
    for r in neg:
        m = M[r]
        i = 0
        if m[1, 1] > m[0, 0]:
            i = 1
        if m[2, 2] > m[i, i]:
            i = 2
        j = (i + 1) % 3
        k = (j + 1) % 3
        t = np.sqrt(m[i, i] - m[j, j] - m[k, k] + 1.0)
        v = np.zeros(3)
        v[i] = 0.5 * t
        s = 0.5 / t
        w = (m[k, j] - m[j, k]) * s
        v[j] = (m[j, i] + m[i, j]) * s
        v[k] = (m[k, i] + m[i, k]) * s
        q[r] = (w, v[0], v[1], v[2])
    return q.reshape(shp + (4,))


# ---------------------------------------------------------- SH rotation ----

def sh_rotation_matrices(R):
    """Real-SH rotation blocks for bands 1..3 from row-major rotations R [N,3,3].

    Returns [sh1 [N,3,3], sh2 [N,5,5], sh3 [N,7,7]] with band-1 ordering
    (y, z, x) as in helper.cpp:988-996."""
    R = np.asarray(R, F64).reshape(-1, 3, 3)
    N = R.shape[0]
    perm = [1, 2, 0]
    b1 = np.empty((N, 3, 3), F64)
    for a in range(3):
        for b in range(3):
            b1[:, a, b] = R[:, perm[a], perm[b]]
    bands = [b1]

    def R1(i, j):          # i,j in -1..1
        return b1[:, i + 1, j + 1]

    for l in range(2, 4):
        prev = bands[-1]
        lp = l - 1

        def Rp(a, b):      # a,b in -(l-1)..(l-1)
            return prev[:, a + lp, b + lp]

        def P(i, a, b):
            if b == l:
                return R1(i, 1) * Rp(a, l - 1) - R1(i, -1) * Rp(a, -l + 1)
            if b == -l:
                return R1(i, 1) * Rp(a, -l + 1) + R1(i, -1) * Rp(a, l - 1)
            return R1(i, 0) * Rp(a, b)

        M = np.zeros((N, 2 * l + 1, 2 * l + 1), F64)
        for m in range(-l, l + 1):
            for n in range(-l, l + 1):
                d = 1.0 if m == 0 else 0.0
                den = float((l + n) * (l - n)) if abs(n) < l else float(2 * l * (2 * l - 1))
                u = np.sqrt((l + m) * (l - m) / den)
                v = 0.5 * np.sqrt((1 + d) * (l + abs(m) - 1) * (l + abs(m)) / den) * (1 - 2 * d)
                w = -0.5 * np.sqrt((l - abs(m) - 1) * (l - abs(m)) / den) * (1 - d)
                acc = np.zeros(N, F64)
                if u != 0:
                    acc += u * P(0, m, n)
                if v != 0:
                    if m == 0:
                        V = P(1, 1, n) + P(-1, -1, n)
                    elif m > 0:
                        V = P(1, m - 1, n) * np.sqrt(1 + (m == 1)) - P(-1, -m + 1, n) * (1 - (m == 1))
                    else:
                        V = P(1, m + 1, n) * (1 - (m == -1)) + P(-1, -m - 1, n) * np.sqrt(1 + (m == -1))
                    acc += v * V
                if w != 0:
                    if m > 0:
                        W = P(1, m + 1, n) + P(-1, -m - 1, n)
                    else:
                        W = P(1, m - 1, n) - P(-1, -m + 1, n)
                    acc += w * W
                M[:, m + l, n + l] = acc
        bands.append(M)
    return bands


_ODD = np.array([1 if (k % 2 == 1) else 0 for k in range(16)], bool)


def rotate_sh(shs, R, flip_odd=True):
    """Rotate interleaved SH [N,48] by rotations R [N,3,3].

    With ``flip_odd`` the odd coefficients are negated before and after the
    band rotation (GaussianView.cpp:3138-3154, cudakdtree.cu:160-196)."""
    s = np.asarray(shs, F64).reshape(-1, 16, 3).copy()
    if flip_odd:
        s[:, _ODD, :] *= -1.0
    sh1, sh2, sh3 = sh_rotation_matrices(R)
    s[:, 1:4] = np.einsum("nij,njc->nic", sh1, s[:, 1:4])
    s[:, 4:9] = np.einsum("nij,njc->nic", sh2, s[:, 4:9])
    s[:, 9:16] = np.einsum("nij,njc->nic", sh3, s[:, 9:16])
    if flip_odd:
        s[:, _ODD, :] *= -1.0
    return s.reshape(-1, 48)


# ------------------------------------------------------ Gaussian refit ----

def end_points(pos, rot, scale):
    """GetEndPoints (GaussianView.cpp:4643-4668): [N,6,3] float32 ordered
    (+axis0, -axis0, +axis1, -axis1, +axis2, -axis2)."""
    R = quat_to_matrix(quat_normalize(rot))
    half = ((np.asarray(scale, F32) + AXIS_PADDING) * END_COEFF).astype(F64)   # [N,3]
    out = np.empty((pos.shape[0], 6, 3), F32)
    p = np.asarray(pos, F32).astype(F64)
    for a in range(3):
        e = R[:, :, a] * half[:, a:a + 1]
        out[:, 2 * a] = (p + e).astype(F32)
        out[:, 2 * a + 1] = (p - e).astype(F32)
    return out


def polar_svd(M):
    """getOthogonalMatrixWithK (helper.cpp:429-440): R = U V^T and
    K = diag(V S V^T) from an SVD in float64."""
    U, S, Vt = np.linalg.svd(np.asarray(M, F64))
    R = U @ Vt
    K = np.einsum("nji,nj,nji->ni", Vt, S, Vt)
    return R, K


def refit_gaussians(ends, rot_old, scale0, shs, static=None):
    """UpdateAsSixPointsWithdrawBad (GaussianView.cpp:3081-3166).

    ends [N,6,3] float32 (already deformed), rot_old [N,4] (the quaternion
    before this frame), scale0 [N,3] (scale_backup_vector), shs [N,48].
    Returns (pos, rot, scale, shs) float32; static Gaussians keep rot_old,
    shs and get pos/scale = None-marked (caller keeps its own)."""
    E = np.asarray(ends, F32).astype(F64)
    N = E.shape[0]
    center = E.mean(axis=1)
    M = np.empty((N, 3, 3), F64)
    for a in range(3):
        M[:, :, a] = 0.5 * (E[:, 2 * a] - E[:, 2 * a + 1])
    M = M.astype(F32).astype(F64)
    R, K = polar_svd(M)
    R = R.astype(F32).astype(F64)
    K = K.astype(F32)
    q = quat_normalize(quat_from_matrix(R)).astype(F32)
    s0 = np.asarray(scale0, F32)
    scale = (K / ((s0 + AXIS_PADDING) * END_COEFF) * s0).astype(F32)
    qo = np.asarray(rot_old, F32).astype(F64)
    qr = quat_normalize(quat_mul(q.astype(F64), quat_inverse(qo)))
    shs_new = rotate_sh(shs, quat_to_matrix(qr)).astype(F32)
    pos = center.astype(F32)
    if static is not None:
        st = np.asarray(static, bool)
        q[st] = np.asarray(rot_old, F32)[st]
        shs_new[st] = np.asarray(shs, F32)[st]
    return pos, q, scale, shs_new


def covariance6(rot, scale):
    """Sigma = R diag(s)^2 R^T packed (xx, xy, xz, yy, yz, zz), float64."""
    R = quat_to_matrix(quat_normalize(rot))
    s2 = np.asarray(scale, F64) ** 2
    S = np.einsum("nij,nj,nkj->nik", R, s2, R)
    return np.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], axis=1)


def skin_gaussians(ends, ends_idx, ends_w, rot_node, trans_node, node_pos,
                   rot_old, scale0, shs, static=None, float_accumulate=True):
    """One frame of Gaussian skinning: ED blend of the 6 endpoints
    (GaussianView.cpp:3022-3040) then the refit.  ``ends_idx``/``ends_w`` are
    [N*6,k] in endpoint order.  Returns (ends_new, pos, rot, scale, shs)."""
    N = ends.shape[0]
    e_new = _ed.ed_blend(ends.reshape(-1, 3), ends_idx, ends_w, rot_node,
                         trans_node, node_pos, float_accumulate).reshape(N, 6, 3)
    pos, q, s, sh = refit_gaussians(e_new, rot_old, scale0, shs, static)
    return (e_new,) + (pos, q, s, sh)


# ------------------------------------------------------------ samples -----

def _inverse3_f64(M):
    return np.linalg.inv(M)


def node_quaternions(rot_node):
    """FastUpdateSamplesSH's per-node part (GaussianView.cpp:3172-3181):
    Newton polar iteration M <- (M + M^-T)/2 until max|dM| < 1e-6
    (helper.cpp:506-517, returns the iterate before the final update), then a
    normalised quaternion (w,x,y,z) float32."""
    n = rot_node.shape[0]
    M = np.asarray(rot_node, F64).reshape(n, 3, 3).transpose(0, 2, 1)  # col-major -> row-major
    M = M.astype(F32).astype(F64)
    active = np.ones(n, bool)
    for _ in range(200):
        if not active.any():
            break
        Ma = M[active]
        nxt = 0.5 * (Ma + np.linalg.inv(Ma).transpose(0, 2, 1))
        done = np.abs(Ma - nxt).max(axis=(1, 2)) < 1e-6
        idx = np.flatnonzero(active)
        upd = idx[~done]
        M[upd] = nxt[~done]
        active[idx[done]] = False
    q = quat_normalize(quat_from_matrix(M)).astype(F32)
    return q


def slerp_blend(idx, w, quats):
    """RotateSHs' quaternion blend (cudakdtree.cu:113-148, 208-217): iterative
    slerp from identity with t = w_j / (w_j + sum of earlier w).  idx [S,k],
    w float32 [S,k], quats (w,x,y,z) float32 [n,4].  Returns float64 [S,4]."""
    S, k = idx.shape
    wf = np.asarray(w, F32)
    cur = np.zeros((S, 4), F64)
    cur[:, 0] = 1.0
    last = np.zeros(S, F32)
    for j in range(k):
        cw = wf[:, j]
        t = (cw / (cw + last)).astype(F64)
        e = np.asarray(quats, F32)[idx[:, j]].astype(F64)
        c32 = cur.astype(F32)
        e32 = e.astype(F32)
        # float32 dot in the reference's (x,y,z,w) order
        cos = ((c32[:, 1] * e32[:, 1] + c32[:, 2] * e32[:, 2]) + c32[:, 3] * e32[:, 3]) + c32[:, 0] * e32[:, 0]
        cos = cos.astype(F32).astype(F64)
        neg = cos < 0
        e[neg] *= -1.0
        cos = np.abs(cos)
        lin = cos > F64(F32(0.99995))
        sin_a = np.sqrt(np.maximum(1.0 - cos * cos, 0.0))
        ang = np.arctan2(sin_a, cos)
        with np.errstate(divide="ignore", invalid="ignore"):
            ra = np.where(lin, 1.0 - t, np.sin((1.0 - t) * ang) / sin_a)
            rb = np.where(lin, t, np.sin(t * ang) / sin_a)
        cur = ra[:, None] * c32.astype(F64) + rb[:, None] * e
        cur = quat_normalize(cur.astype(F32).astype(F64))
        last = (last + cw).astype(F32)
    return cur


def skin_samples(sample_pos, idx, w, rot_node, trans_node, node_pos, feature,
                 static=None, float_accumulate=True):
    """UpdatePositionforSamples (GaussianView.cpp:3060-3077) and
    FastUpdateSamplesSH (GaussianView.cpp:3169-3186).  Returns (pos, feature)."""
    pos = _ed.ed_blend(sample_pos, idx, np.asarray(w, F64), rot_node, trans_node, node_pos,
                       float_accumulate)
    q = node_quaternions(rot_node)
    qb = slerp_blend(idx, np.asarray(w, F32), q)
    feat = rotate_sh(feature, quat_to_matrix(quat_normalize(qb))).astype(F32)
    if static is not None:
        st = np.asarray(static, bool)
        pos[st] = np.asarray(sample_pos, F32)[st]
        feat[st] = np.asarray(feature, F32)[st]
    return pos, feat


def static_mask(idx, static_nodes, n_nodes):
    """An item is static when all its k neighbour nodes are static
    (GaussianView.cpp:2040-2066)."""
    is_static = np.zeros(n_nodes, bool)
    is_static[np.asarray(static_nodes, np.int64)] = True
    return is_static[idx].all(axis=1)


# ------------------------------------------------------------- adjoint ----

def skin_forward_from_nodes(ends_in, idx, w, X, node_pos, scale0):
    """(mu, Sigma [N,3,3]) of the skinned Gaussians as a function of the node
    transforms X [n,12] ([R column-major | t]), float64 throughout; idx/w are
    Gaussian-major [N*6, k]."""
    n = X.shape[0]
    N = ends_in.shape[0]
    R = X[:, :9].reshape(n, 3, 3).transpose(0, 2, 1)
    t = X[:, 9:]
    g = np.asarray(node_pos, F64)
    P = np.asarray(ends_in, F64).reshape(-1, 3)
    out = np.zeros_like(P)
    for j in range(idx.shape[1]):
        nj = idx[:, j]
        out += np.asarray(w, F64)[:, j:j + 1] * (np.einsum("nij,nj->ni", R[nj], P - g[nj]) + g[nj] + t[nj])
    P2 = out.reshape(N, 6, 3)
    mu = P2.mean(1)
    M = np.stack([(P2[:, 2 * a] - P2[:, 2 * a + 1]) / 2 for a in range(3)], axis=2)
    U, S, Vt = np.linalg.svd(M)
    Rp = U @ Vt
    K = np.einsum("nra,nra->na", Rp, M)
    s0 = np.asarray(scale0, F64)
    s = s0 / ((s0 + 1e-3) * 2) * K
    Sig = np.einsum("nia,na,nja->nij", Rp, s * s, Rp)
    return mu, Sig


def skin_backward(ends_in, idx, w, X, node_pos, scale0, g_mu, g_sigma):
    """dL/dX [n,12] for L = sum g_mu . mu + sum g_sigma : Sigma (g_sigma
    symmetric [N,3,3]), float64, by the chain rule through the polar factor
    (M = R S: dR = R [w]x, (tr S I - S) w = skew(R^T dM))."""
    n = X.shape[0]
    N = ends_in.shape[0]
    g = np.asarray(node_pos, F64)
    R = X[:, :9].reshape(n, 3, 3).transpose(0, 2, 1)
    t = X[:, 9:]
    P = np.asarray(ends_in, F64).reshape(-1, 3)
    wf = np.asarray(w, F64)
    out = np.zeros_like(P)
    for j in range(idx.shape[1]):
        nj = idx[:, j]
        out += wf[:, j:j + 1] * (np.einsum("nij,nj->ni", R[nj], P - g[nj]) + g[nj] + t[nj])
    P2 = out.reshape(N, 6, 3)
    M = np.stack([(P2[:, 2 * a] - P2[:, 2 * a + 1]) / 2 for a in range(3)], axis=2)
    U, _, Vt = np.linalg.svd(M)
    Rp = U @ Vt
    Sm = np.einsum("nra,nrb->nab", Rp, M)
    Sm = 0.5 * (Sm + Sm.transpose(0, 2, 1))
    K = np.einsum("naa->na", Sm)
    s0 = np.asarray(scale0, F64)
    c = s0 / ((s0 + 1e-3) * 2)
    D = (c * K) ** 2
    G = np.asarray(g_sigma, F64)
    gR = 2 * np.einsum("nij,njk,nk->nik", G, Rp, D)
    gK = np.einsum("nia,nij,nja->na", Rp, G, Rp) * 2 * c * c * K
    gM = Rp * gK[:, None, :]
    gR = gR + M * gK[:, None, :]
    A = np.einsum("nri,nrj->nij", Rp, gR)
    a = 0.5 * np.stack([A[:, 2, 1] - A[:, 1, 2], A[:, 0, 2] - A[:, 2, 0], A[:, 1, 0] - A[:, 0, 1]], 1)
    T = np.einsum("nii->n", Sm)[:, None, None] * np.eye(3) - Sm
    om = np.linalg.solve(T, a[..., None])[..., 0]
    Y = np.zeros((N, 3, 3))
    Y[:, 0, 1], Y[:, 0, 2], Y[:, 1, 2] = -om[:, 2], om[:, 1], -om[:, 0]
    Y[:, 1, 0], Y[:, 2, 0], Y[:, 2, 1] = om[:, 2], -om[:, 1], om[:, 0]
    gM = gM + 2 * np.einsum("nij,njk->nik", Rp, Y)
    gP = np.repeat(np.asarray(g_mu, F64)[:, None, :] / 6, 6, 1)
    for q in range(3):
        gP[:, 2 * q] += gM[:, :, q] / 2
        gP[:, 2 * q + 1] -= gM[:, :, q] / 2
    gP = gP.reshape(-1, 3)
    gX = np.zeros((n, 12))
    for j in range(idx.shape[1]):
        nj = idx[:, j]
        d = P - g[nj]
        contrib = wf[:, j:j + 1, None] * gP[:, :, None] * d[:, None, :]
        np.add.at(gX, (nj, slice(0, 9)), contrib.transpose(0, 2, 1).reshape(-1, 9))
        np.add.at(gX, (nj, slice(9, 12)), wf[:, j:j + 1] * gP)
    return gX


def packed_to_sym(g6):
    """Upstream gradient of packed (xx,xy,xz,yy,yz,zz) as the symmetric G with
    dL = sum G : dSigma."""
    g6 = np.asarray(g6, F64)
    G = np.empty((g6.shape[0], 3, 3))
    G[:, 0, 0], G[:, 1, 1], G[:, 2, 2] = g6[:, 0], g6[:, 3], g6[:, 5]
    G[:, 0, 1] = G[:, 1, 0] = 0.5 * g6[:, 1]
    G[:, 0, 2] = G[:, 2, 0] = 0.5 * g6[:, 2]
    G[:, 1, 2] = G[:, 2, 1] = 0.5 * g6[:, 4]
    return G
