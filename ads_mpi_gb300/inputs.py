"""Seeded synthetic inputs of the benchmark configurations.

No dataset is involved: every field is generated on the host in FP64 from a
numpy ``default_rng(seed)`` and evaluated at the quadrature points, so the CPU
oracle and the GPU path see bit-identical inputs.  Arrays use the per-point
layout of the C-ABI, (kx,ky,kz,ex,ey,ez) column-major = numpy C-order shape
(Ez, Ey, Ex, q, q, q).
"""
import numpy as np


def projection_target(x, y, z, seed=0):
    """L2-projection target: sin(2 pi x) sin(2 pi y) sin(2 pi z) plus
    0.1 * sum_{k=1..8} a_k exp(-|x - c_k|^2 / 0.01), a_k ~ U(-1,1), c_k ~ U[0,1]^3."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1.0, 1.0, 8)
    c = rng.uniform(0.0, 1.0, (8, 3))
    f = np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)
    for k in range(8):
        r2 = (x - c[k, 0]) ** 2 + (y - c[k, 1]) ** 2 + (z - c[k, 2]) ** 2
        f = f + 0.1 * a[k] * np.exp(-r2 / 0.01)
    return np.ascontiguousarray(f, dtype=np.float64)


def gaussian_bumps(x, y, z, seed=0, n=16, width=0.05):
    """Heat initial state: sum of n Gaussian bumps A_i exp(-|x - c_i|^2 / (2 width^2)),
    A_i ~ U(0,1), c_i ~ U[0.2,0.8]^3 (width is the standard deviation)."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.0, 1.0, n)
    c = rng.uniform(0.2, 0.8, (n, 3))
    f = np.zeros(np.broadcast(x, y, z).shape)
    for i in range(n):
        r2 = (x - c[i, 0]) ** 2 + (y - c[i, 1]) ** 2 + (z - c[i, 2]) ** 2
        f = f + A[i] * np.exp(-r2 / (2.0 * width * width))
    return np.ascontiguousarray(f, dtype=np.float64)


def _grf_grid(seed, sigma, corr, grid):
    """The field of gaussian_random_field on its grid^3 mesh (cell vertices i/grid)."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((grid, grid, grid))
    k = np.fft.fftfreq(grid, d=1.0 / grid) * 2 * np.pi
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    # square root of the spectral density of the squared-exponential kernel
    amp = np.exp(-0.25 * corr * corr * (kx * kx + ky * ky + kz * kz))
    g = np.real(np.fft.ifftn(np.fft.fftn(noise) * amp))
    g = g - g.mean()
    return g * (sigma / g.std())


def _trilinear_weights(X, grid):
    """Dense (points, grid) matrix of the periodic linear interpolation weights."""
    x = np.asarray(X, dtype=np.float64).reshape(-1) * grid
    i0 = np.floor(x).astype(np.int64)
    f = x - i0
    W = np.zeros((x.size, grid))
    r = np.arange(x.size)
    np.add.at(W, (r, i0 % grid), 1.0 - f)
    np.add.at(W, (r, (i0 + 1) % grid), f)
    return W


def gaussian_random_field_qp(Xx, Xy, Xz, seed=0, sigma=0.5, corr=0.1, grid=64, device=None):
    """gaussian_random_field on the tensor grid of quadrature points: the same
    field and trilinear interpolation, applied axis by axis (the weights are
    separable).  Xx, Xy, Xz are the per-axis point tables (E, q); the result has
    the per-point layout shape (Ez, Ey, Ex, q, q, q).  Uses torch on `device`
    when given."""
    g = _grf_grid(seed, sigma, corr, grid)
    Wx, Wy, Wz = (_trilinear_weights(X, grid) for X in (Xx, Xy, Xz))
    Ex, q = np.asarray(Xx).shape
    Ey, Ez = np.asarray(Xy).shape[0], np.asarray(Xz).shape[0]
    if device is not None:
        import torch
        tg = torch.as_tensor(g, device=device)
        wx, wy, wz = (torch.as_tensor(W, device=device) for W in (Wx, Wy, Wz))
        t = torch.einsum("ai,ijk->ajk", wx, tg)
        t = torch.einsum("bj,ajk->abk", wy, t)
        t = torch.einsum("ck,abk->cba", wz, t)          # (QZ, QY, QX)
        t = t.reshape(Ez, q, Ey, q, Ex, q).permute(0, 2, 4, 1, 3, 5).contiguous()
        return t.cpu().numpy()
    t = np.einsum("ai,ijk->ajk", Wx, g)
    t = np.einsum("bj,ajk->abk", Wy, t)
    t = np.einsum("ck,abk->cba", Wz, t)
    return np.ascontiguousarray(t.reshape(Ez, q, Ey, q, Ex, q).transpose(0, 2, 4, 1, 3, 5))


def gaussian_random_field(x, y, z, seed=0, sigma=0.5, corr=0.1, grid=64):
    """Stationary Gaussian random field with squared-exponential covariance
    sigma^2 exp(-|r|^2 / (2 corr^2)) on the periodic unit cube: white noise is
    filtered in Fourier space on a uniform `grid`^3 mesh, normalised to variance
    sigma^2, and evaluated at (x, y, z) by trilinear interpolation."""
    g = _grf_grid(seed, sigma, corr, grid)
    # trilinear interpolation on the periodic grid (cell-vertex at i/grid)
    X = np.asarray(x) * grid
    Y = np.asarray(y) * grid
    Z = np.asarray(z) * grid
    shape = np.broadcast(X, Y, Z).shape
    X, Y, Z = (np.broadcast_to(v, shape) for v in (X, Y, Z))
    i0 = np.floor(X).astype(np.int64)
    j0 = np.floor(Y).astype(np.int64)
    k0 = np.floor(Z).astype(np.int64)
    fx, fy, fz = X - i0, Y - j0, Z - k0
    out = np.zeros(shape)
    for di in (0, 1):
        wx = fx if di else 1.0 - fx
        ii = (i0 + di) % grid
        for dj in (0, 1):
            wy = fy if dj else 1.0 - fy
            jj = (j0 + dj) % grid
            for dk in (0, 1):
                wz = fz if dk else 1.0 - fz
                kk = (k0 + dk) % grid
                out += wx * wy * wz * g[ii, jj, kk]
    return np.ascontiguousarray(out, dtype=np.float64)


def gaussian_bumps_separable(Xx, Xy, Xz, seed=0, n=16, width=0.05, device=None):
    """gaussian_bumps on the tensor grid of quadrature points, using that each
    bump factors per axis: exp(-|x-c|^2/(2w^2)) = gx(x) gy(y) gz(z).  Xx, Xy, Xz
    are the per-axis point tables (E, q); the result has the per-point layout
    shape (Ez, Ey, Ex, q, q, q).  Uses torch on `device` when given (fast at
    256^3), numpy otherwise; the bump parameters are drawn exactly as in
    gaussian_bumps."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.0, 1.0, n)
    c = rng.uniform(0.2, 0.8, (n, 3))
    s2 = 2.0 * width * width
    if device is not None:
        import torch
        tx = torch.as_tensor(Xx, dtype=torch.float64, device=device)
        ty = torch.as_tensor(Xy, dtype=torch.float64, device=device)
        tz = torch.as_tensor(Xz, dtype=torch.float64, device=device)
        Ez, q = tz.shape
        Ey, Ex = ty.shape[0], tx.shape[0]
        out = torch.zeros((Ez, Ey, Ex, q, q, q), dtype=torch.float64, device=device)
        for i in range(n):
            gx = torch.exp(-(tx - float(c[i, 0])) ** 2 / s2)
            gy = torch.exp(-(ty - float(c[i, 1])) ** 2 / s2)
            gz = torch.exp(-(tz - float(c[i, 2])) ** 2 / s2) * float(A[i])
            yz = gz[:, None, :, None] * gy[None, :, None, :]           # (Ez, Ey, qz, qy)
            out += yz[:, :, None, :, :, None] * gx[None, None, :, None, None, :]
        return out.cpu().numpy()
    Ez, q = Xz.shape
    out = np.zeros((Xz.shape[0], Xy.shape[0], Xx.shape[0], q, q, q))
    for i in range(n):
        gx = np.exp(-(Xx - c[i, 0]) ** 2 / s2)
        gy = np.exp(-(Xy - c[i, 1]) ** 2 / s2)
        gz = np.exp(-(Xz - c[i, 2]) ** 2 / s2) * A[i]
        yz = gz[:, None, :, None] * gy[None, :, None, :]
        out += yz[:, :, None, :, :, None] * gx[None, None, :, None, None, :]
    return out


# ---------------------------------------------------------------------------
# The oil problem's pointwise data (problems/oil/input_data.F90).  The
# reference draws its curves with Fortran random_number and reads the pump and
# drain positions from the command line; here both come from seeded numpy
# generators.  The functions restate falloff/lerp/bump3d (src/math.F90:44-88,
# 173-181), dist_from_segment/dist_from_curves (input_data.F90:166-237),
# pumping/draining (:241-283), kq (:286-294) and initial_state (:307-318).
# ---------------------------------------------------------------------------
OIL_RADIUS = 0.15
OIL_KQMIN, OIL_KQMAX = 1.0, 1000.0


def _falloff(r, R, t):
    h = (t - r) / (R - r)
    v = ((h - 1.0) * (h + 1.0)) ** 2
    return np.where(t < r, 1.0, np.where(t > R, 0.0, v))


def _lerp(t, x, y):
    return (1.0 - t) * x + t * y


def oil_curves(seed=0, cN=30, cL=16, step=0.05):
    """The cN random-walk curves of cL points each (InitInputData,
    input_data.F90:137-163): a random start and direction, then cL - 1 steps
    whose direction is nudged by a random acceleration.  Shape (cN, cL, 3)."""
    rng = np.random.default_rng(seed)
    c = np.zeros((cN, cL, 3))
    for i in range(cN):
        c[i, 0] = rng.random(3)
        dx = rng.random(3)
        for j in range(1, cL):
            rng.random(3)  # the reference draws t here and does not use it
            ddx = rng.random(3)
            ddx = 2.0 * (ddx - 0.5) - 0.4 * dx * np.sum(dx ** 2)
            dx = dx + 0.4 * ddx
            c[i, j] = c[i, j - 1] + step * dx
    return c


def oil_wells(seed=0, npumps=2, ndrains=2):
    """Pump and drain positions (InitPumps reads them from the command line)."""
    rng = np.random.default_rng(seed + 1)
    return rng.uniform(0.2, 0.8, (npumps, 3)), rng.uniform(0.2, 0.8, (ndrains, 3))


def _dist2_from_curves(P, curves, chunk=4096):
    """Squared distance of each point of P (M, 3) to the nearest curve segment,
    starting from 1e3 as the reference does."""
    a = curves[:, :-1].reshape(-1, 3)
    b = curves[:, 1:].reshape(-1, 3)
    d = b - a
    len2 = np.sum(d * d, axis=1)
    out = np.empty(P.shape[0])
    for s in range(0, P.shape[0], chunk):
        p = P[s:s + chunk, None, :]
        c = p - a[None]
        proj = np.sum(c * d[None], axis=2) / len2[None]
        near = np.where((proj < 0.0)[..., None], a[None],
                        np.where((proj > 1.0)[..., None], b[None], a[None] + proj[..., None] * d[None]))
        out[s:s + chunk] = np.minimum(1e3, np.min(np.sum((p - near) ** 2, axis=2), axis=1))
    return out


def _oil_fields_torch(x, y, z, curves, pumps, drains, device, chunk=1 << 17):
    """oil_fields on a torch device, the same formulas in FP64."""
    import torch

    def t(v):
        return torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=device)

    def falloff(r, R, d):
        h = (d - r) / (R - r)
        v = ((h - 1.0) * (h + 1.0)) ** 2
        return torch.where(d < r, torch.ones_like(d), torch.where(d > R, torch.zeros_like(d), v))

    shape = np.broadcast(x, y, z).shape
    P = torch.stack([t(np.broadcast_to(v, shape)).reshape(-1) for v in (x, y, z)], dim=1)
    a, b = t(curves[:, :-1].reshape(-1, 3)), t(curves[:, 1:].reshape(-1, 3))
    d = b - a
    len2 = (d * d).sum(dim=1)
    d2 = torch.empty(P.shape[0], dtype=torch.float64, device=device)
    for s in range(0, P.shape[0], chunk):
        p = P[s:s + chunk, None, :]
        proj = ((p - a[None]) * d[None]).sum(dim=2) / len2[None]
        near = torch.where((proj < 0.0)[..., None], a[None],
                           torch.where((proj > 1.0)[..., None], b[None], a[None] + proj[..., None] * d[None]))
        d2[s:s + chunk] = torch.clamp(((p - near) ** 2).sum(dim=2).min(dim=1).values, max=1e3)
    dist = torch.sqrt(d2)
    kq = (1.0 - falloff(0.0, 0.06, dist)) * OIL_KQMIN + falloff(0.0, 0.06, dist) * OIL_KQMAX
    pump = sum(falloff(0.0, OIL_RADIUS, torch.linalg.norm(t(w)[None] - P, dim=1)) for w in pumps)
    drain = sum(falloff(0.0, OIL_RADIUS, torch.linalg.norm(t(w)[None] - P, dim=1)) for w in drains)
    bump = falloff(0.2 / 2.0, 0.6 / 2.0, torch.linalg.norm(P - 0.5, dim=1))
    init = 0.1 * falloff(0.0, 0.1, dist) * bump
    return {k: v.reshape(shape).cpu().numpy() for k, v in
            (("kq", kq), ("pump", pump), ("drain", drain), ("init", init))}


def oil_fields(x, y, z, seed=0, npumps=2, ndrains=2, device=None):
    """Kq, pumping, the draining weight w (draining(u, X) = w u) and the
    initial state at the points (x, y, z); arrays of the points' shape.  Uses
    torch on `device` when given (large grids), numpy otherwise."""
    shape = np.broadcast(x, y, z).shape
    curves = oil_curves(seed)
    pumps, drains = oil_wells(seed, npumps, ndrains)
    if device is not None:
        return _oil_fields_torch(x, y, z, curves, pumps, drains, device)
    P = np.stack([np.broadcast_to(v, shape).ravel() for v in (x, y, z)], axis=1)
    dist = np.sqrt(_dist2_from_curves(P, curves))
    kq = _lerp(_falloff(0.0, 0.06, dist), OIL_KQMIN, OIL_KQMAX)
    pump = np.zeros(P.shape[0])
    for i in range(npumps):
        pump += _falloff(0.0, OIL_RADIUS, np.linalg.norm(pumps[i][None] - P, axis=1))
    drain = np.zeros(P.shape[0])
    for i in range(ndrains):
        drain += _falloff(0.0, OIL_RADIUS, np.linalg.norm(drains[i][None] - P, axis=1))
    bump = _falloff(0.2 / 2.0, 0.6 / 2.0, np.linalg.norm(P - 0.5, axis=1))
    init = 0.1 * _lerp(_falloff(0.0, 0.1, dist), 0.0, 1.0) * bump
    return {k: np.ascontiguousarray(v.reshape(shape)) for k, v in
            (("kq", kq), ("pump", pump), ("drain", drain), ("init", init))}
