"""Environment-grid operators of the oracle (NumPy restatements).

Each function restates one reference helper; the grid is row-major
``(ny, nx)`` exactly as ``FiniteDiffSolver.cell_grid`` lays it out
(``betse/science/math/finitediff.py:158-250``, ``k = i*nx + j``).
"""
from __future__ import annotations

import numpy as np


def gradient(F, delx, dely=None):
    """``fd.gradient`` (finitediff.py:1236-1266): central differences inside,
    one-sided differences on the four edges."""
    if dely is None:
        dely = delx
    dFx = np.zeros(F.shape)
    dFy = np.zeros(F.shape)
    dFx[:, 1:-1] = -(F[:, :-2] - F[:, 2:]) / (2 * delx)
    dFy[1:-1, :] = -(F[:-2, :] - F[2:, :]) / (2 * dely)
    dFx[:, 0] = (F[:, 1] - F[:, 0]) / delx
    dFx[:, -1] = (F[:, -1] - F[:, -2]) / delx
    dFy[0, :] = (F[1, :] - F[0, :]) / dely
    dFy[-1, :] = (F[-1, :] - F[-2, :]) / dely
    return dFx, dFy


def diff(F, delx, axis=0):
    """``fd.diff`` (finitediff.py:1268-1303). The one-sided edge terms carry the
    reference's flipped signs (``:1276-1277, :1292-1293``) on purpose."""
    dF = np.zeros(F.shape)
    if axis == 1:
        dF[1:-1, :] = -(F[:-2, :] - F[2:, :]) / (2 * delx)
        dF[0, :] = -(F[1, :] - F[0, :]) / delx
        dF[-1, :] = -(F[-1, :] - F[-2, :]) / delx
    else:
        dF[:, 1:-1] = -(F[:, :-2] - F[:, 2:]) / (2 * delx)
        dF[:, 0] = (F[:, 0] - F[:, 1]) / delx
        dF[:, -1] = (F[:, -2] - F[:, -1]) / delx
    return dF


def divergence(Fx, Fy, delx, dely):
    """``fd.divergence`` (finitediff.py:1305-1311)."""
    return diff(Fx, delx, axis=0) + diff(Fy, dely, axis=1)


def integrator(P, sharp=0.5):
    """``fd.integrator`` (finitediff.py:1479-1512): nearest-neighbour blend,
    edges kept."""
    F = np.zeros(P.shape)
    sides = (1 - sharp) / 4
    F[:, :] = sharp * P
    F[0:-1, :] += sides * P[1:, :]
    F[1:, :] += sides * P[0:-1, :]
    F[:, 0:-1] += sides * P[:, 1:]
    F[:, 1:] += sides * P[:, 0:-1]
    F[:, 0] = P[:, 0]
    F[:, -1] = P[:, -1]
    F[0, :] = P[0, :]
    F[-1, :] = P[-1, :]
    return F


def gaussian_kernel(sigma=1.0, truncate=4.0):
    """The normalised 1-D Gaussian that ``scipy.ndimage.gaussian_filter`` uses
    (radius ``int(truncate*sigma + 0.5)``)."""
    r = int(truncate * sigma + 0.5)
    x = np.arange(-r, r + 1, dtype=np.float64)
    w = np.exp(-0.5 / (sigma * sigma) * x * x)
    return w / w.sum(), r


def gaussian_filter(a, sigma=1.0, mode='reflect', cval=0.0):
    """Separable Gaussian, axis 0 then axis 1, as scipy applies it.

    ``mode='reflect'`` is scipy's half-sample symmetric extension (numpy's
    ``'symmetric'`` pad); ``mode='constant'`` pads with ``cval``. Used by
    ``get_current`` (``betse/science/physics/ion_current.py:94,130``).
    """
    w, r = gaussian_kernel(sigma)
    out = np.asarray(a, np.float64)
    for axis in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[axis] = (r, r)
        if mode == 'constant':
            ap = np.pad(out, pad, mode='constant', constant_values=cval)
        else:
            ap = np.pad(out, pad, mode='symmetric')
        n = out.shape[axis]
        acc = np.zeros(out.shape)
        for k in range(2 * r + 1):
            sl = [slice(None), slice(None)]
            sl[axis] = slice(k, k + n)
            acc += w[k] * ap[tuple(sl)]
        out = acc
    return out


def make_laplacian(ny, nx, delta):
    """``FiniteDiffSolver.makeLaplacian`` with all four edges ``'value'``
    (finitediff.py:252-431, called at cells.py:503): 5-point stencil inside,
    identity rows on the edges, all divided by delta**2."""
    G = ny * nx
    A = np.zeros((G, G))
    k = np.arange(G)
    i, j = k // nx, k % nx
    inner = (i > 0) & (i < ny - 1) & (j > 0) & (j < nx - 1)
    ki = k[inner]
    A[ki, ki] = -4.0
    A[ki, ki + nx] = 1.0
    A[ki, ki - nx] = 1.0
    A[ki, ki + 1] = 1.0
    A[ki, ki - 1] = 1.0
    kb = k[~inner]
    A[kb, kb] = 1.0
    return A / (delta ** 2)


def make_laplacian_inverse(ny, nx, delta):
    """``lapENVinv``: the reference takes ``np.linalg.pinv`` of the matrix
    above; it is non-singular, so the inverse is the same operator."""
    return np.linalg.inv(make_laplacian(ny, nx, delta))


def hh_decomp(JJx, JJy, lap_inv, shape, delta, bounds=None, sigma=1.0):
    """Helmholtz-Hodge split of an environment vector field
    (``sim_toolbox.HH_Decomp``, sim_toolbox.py:1236-1290)."""
    if bounds is not None:
        Lb, Rb, Tb, Bb = bounds['L'], bounds['R'], bounds['T'], bounds['B']
    else:
        Lb = Rb = Tb = Bb = 0.0
    Jxr = -JJy.reshape(shape)
    Jyr = JJx.reshape(shape)
    divJr = divergence(Jxr, Jyr, delta, delta)
    divJr[:, 0] = 0.0
    divJr[:, -1] = 0.0
    divJr[0, :] = 0.0
    divJr[-1, :] = 0.0
    AA = lap_inv @ (-divJr.ravel())
    gAx, gAy = gradient(AA.reshape(shape), delta)
    Fx, Fy = -gAy, gAx
    divJd = divergence(JJx.reshape(shape) / sigma, JJy.reshape(shape) / sigma,
                       delta, delta)
    divJd[:, 0] = -Lb * (1 / delta ** 2)
    divJd[:, -1] = -Rb * (1 / delta ** 2)
    divJd[0, :] = -Bb * (1 / delta ** 2)
    divJd[-1, :] = -Tb * (1 / delta ** 2)
    BB = lap_inv @ divJd.ravel()
    Gx, Gy = gradient(BB.reshape(shape), delta)
    return AA, Fx, Fy, BB, Gx, Gy
