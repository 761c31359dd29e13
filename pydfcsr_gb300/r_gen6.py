"""FP64 6x6 linear transfer matrices (drift / sector bend / quad / roll / edges).

Host-side harness for synthetic beams: the reference imports ``r_gen6`` at
``pyDFCSR_2D/CSR.py:17`` but tracks with bmadx; here the same linear optics
(``pyDFCSR_2D/r_gen6.py:4-122``) carries seeded beams from one wake step to the
next so that the device path and the oracle see identical particles.

Coordinates are (x, x', y, y', z, delta).  The body of a combined-function
sector magnet with curvature h = angle/L and gradient k1 has horizontal
focusing kx^2 = k1 + h^2 and vertical ky^2 = -k1; bend pole faces add thin
edge kicks of strength h*tan(E) (horizontal) and -h*tan(E - psi) (vertical,
psi the fringe-field correction from the half gap).  A roll rotates the body
matrix about the z axis.  The same conventions as the reference are used so
that its known-answer vectors (``test/test_BmadX_tracking.ipynb``) reproduce.
"""
import math

import numpy as np

__all__ = ["r_gen6"]


def _plane(k2, L):
    """2x2 transfer matrix of one transverse plane with focusing k2 over L,
    plus the (cos-like, sin-like, k) terms needed for dispersion."""
    k = math.sqrt(abs(k2))
    phi = k * L
    if abs(phi) < 1.0e-12:
        return np.array([[1.0, L], [0.0, 1.0]]), None
    if k2 > 0:
        c, s = math.cos(phi), math.sin(phi)
        m = np.array([[c, s / k], [-k * s, c]])
    else:
        c, s = math.cosh(phi), math.sinh(phi)
        m = np.array([[c, s / k], [k * s, c]])
    return m, (c, s, k, phi)


def _roll_matrix(roll):
    if not roll:
        return np.eye(6)
    c, s = math.cos(-roll), math.sin(-roll)
    o = np.eye(6)
    o[0, 0] = o[1, 1] = o[2, 2] = o[3, 3] = c
    o[0, 2] = o[1, 3] = s
    o[2, 0] = o[3, 1] = -s
    return o


def r_gen6(L, angle=0.0, k1=0.0, roll=0.0, E1=0.0, E2=0.0, hgap=0.0):
    """Return the 6x6 transfer matrix of one element.

    ``L == 0`` returns the pure roll rotation.  Mirrors the argument meaning of
    ``pyDFCSR_2D/r_gen6.py:4`` (L [m], angle [rad], k1 [1/m^2], roll [rad],
    E1/E2 pole-face angles [rad], hgap half gap [m]).
    """
    rot = _roll_matrix(roll)
    if L == 0:
        return rot
    h = angle / L
    kx2 = k1 + h * h
    body = np.zeros((6, 6))

    mx, tx = _plane(kx2, L)
    body[0:2, 0:2] = mx
    if tx is not None:
        c, s, k, phi = tx
        d0 = h * (1.0 - c) / kx2      # x per unit delta
        d1 = h * s / k                # x' per unit delta
        body[0, 5] = d0
        body[1, 5] = d1
        body[4, 0] = -d1
        body[4, 1] = -d0
        body[4, 5] = -(h * h) * (phi - k * mx[0, 1]) / k ** 3
    my, _ = _plane(-k1, L)
    body[2:4, 2:4] = my
    body[4, 4] = 1.0
    body[5, 5] = 1.0

    out = rot @ body @ rot.T
    if angle:
        def edge(e):
            psi = h * hgap * (1.0 + math.sin(e) ** 2) / math.cos(e)
            m = np.eye(6)
            m[1, 0] = math.tan(e) * h
            m[3, 2] = -math.tan(e - psi) * h
            return m
        out = edge(E2) @ out @ edge(E1)
    return out
