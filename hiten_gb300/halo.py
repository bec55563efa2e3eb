"""Halo-orbit initial guesses (Richardson's third-order approximation),
vectorized over a batch of amplitudes.

Restates algorithms/types/services/orbits.py:1060-1223 with the collinear-
point quantities of algorithms/types/services/libration.py:595-660, 1031-1160:
gamma (distance of L1/L2 from the secondary, root of the quintic), the
Legendre coefficients c_n, and the in-plane frequency lambda of the
linearized motion.  Richardson, D. L. (1980), "Analytic construction of
periodic orbits about the collinear points", Celestial Mechanics 22.

`amplitude_z` is in units of gamma (as in the reference); zenith
'northern' gives delta_n = -1, i.e. z0 < 0 at tau = 0 (reference sign
convention, orbits.py:1050-1058, 1176).
"""
import numpy as np


def gamma(mu, point):
    """Distance of L1 (point=1) or L2 (point=2) from the secondary: the real
    root in (0, 1) of the collinear quintic, polished by Newton's method."""
    if point == 1:
        c = [1.0, -(3.0 - mu), 3.0 - 2.0 * mu, -mu, 2.0 * mu, -mu]
    elif point == 2:
        c = [1.0, 3.0 - mu, 3.0 - 2.0 * mu, -mu, -2.0 * mu, -mu]
    else:
        raise ValueError("halo guesses are defined for L1 and L2")
    roots = np.roots(c)
    real = roots[np.abs(roots.imag) < 1e-9].real
    g = float(real[(real > 0) & (real < 1)][0])
    p = np.poly1d(c)
    dp = p.deriv()
    for _ in range(3):
        g = g - p(g) / dp(g)
    return g


def cn(mu, point, n, g=None):
    """Legendre coefficient c_n of the expansion about L1/L2."""
    g = gamma(mu, point) if g is None else g
    if point == 1:
        return (1.0 / g ** 3) * (mu + (-1) ** n * (1 - mu) * g ** (n + 1) / (1 - g) ** (n + 1))
    return (1.0 / g ** 3) * ((-1) ** n * mu + (-1) ** n * (1 - mu) * g ** (n + 1) / (1 + g) ** (n + 1))


def inplane_frequency(c2):
    """lambda of the linear in-plane oscillation: lambda^4 + (c2-2) lambda^2 - (c2-1)(1+2c2) = 0."""
    return float(np.sqrt(0.5 * ((2.0 - c2) + np.sqrt(9.0 * c2 * c2 - 8.0 * c2))))


def third_order_guess(mu, point, amplitude_z, zenith):
    """(N, 6) initial states of Richardson's third-order halo solution at tau = 0.

    amplitude_z: scalar or (N,) in units of gamma; zenith: 'northern'/'southern'
    scalar or (N,)."""
    Az = np.atleast_1d(np.asarray(amplitude_z, dtype=np.float64))
    zen = np.broadcast_to(np.asarray(zenith), Az.shape)
    deltan = np.where(zen == "northern", -1.0, 1.0)
    g = gamma(mu, point)
    c2, c3, c4 = (cn(mu, point, n, g) for n in (2, 3, 4))
    lam = inplane_frequency(c2)
    k = 2 * lam / (lam ** 2 + 1 - c2)
    delta = lam ** 2 - c2
    d1 = (3 * lam ** 2 / k) * (k * (6 * lam ** 2 - 1) - 2 * lam)
    d2 = (8 * lam ** 2 / k) * (k * (11 * lam ** 2 - 1) - 2 * lam)
    a21 = (3 * c3 * (k ** 2 - 2)) / (4 * (1 + 2 * c2))
    a22 = (3 * c3) / (4 * (1 + 2 * c2))
    a23 = -(3 * c3 * lam / (4 * k * d1)) * (3 * k ** 3 * lam - 6 * k * (k - lam) + 4)
    a24 = -(3 * c3 * lam / (4 * k * d1)) * (2 + 3 * k * lam)
    b21 = -(3 * c3 * lam / (2 * d1)) * (3 * k * lam - 4)
    b22 = (3 * c3 * lam) / d1
    d21 = -c3 / (2 * lam ** 2)
    w = 9 * lam ** 2 + 1
    a31 = (-(9 * lam / (4 * d2)) * (4 * c3 * (k * a23 - b21) + k * c4 * (4 + k ** 2))
           + ((w - c2) / (2 * d2)) * (3 * c3 * (2 * a23 - k * b21) + c4 * (2 + 3 * k ** 2)))
    a32 = -(1 / d2) * ((9 * lam / 4) * (4 * c3 * (k * a24 - b22) + k * c4)
                       + 1.5 * (w - c2) * (c3 * (k * b22 + d21 - 2 * a24) - c4))
    b31 = (0.375 / d2) * (8 * lam * (3 * c3 * (k * b21 - 2 * a23) - c4 * (2 + 3 * k ** 2))
                          + (w + 2 * c2) * (4 * c3 * (k * a23 - b21) + k * c4 * (4 + k ** 2)))
    b32 = (1 / d2) * (9 * lam * (c3 * (k * b22 + d21 - 2 * a24) - c4)
                      + 0.375 * (w + 2 * c2) * (4 * c3 * (k * a24 - b22) + k * c4))
    d31 = (3 / (64 * lam ** 2)) * (4 * c3 * a24 + c4)
    d32 = (3 / (64 * lam ** 2)) * (4 * c3 * (a23 - d21) + c4 * (4 + k ** 2))
    den = 2 * lam * (lam * (1 + k ** 2) - 2 * k)
    s1 = (1 / den) * (1.5 * c3 * (2 * a21 * (k ** 2 - 2) - a23 * (k ** 2 + 2) - 2 * k * b21)
                      - 0.375 * c4 * (3 * k ** 4 - 8 * k ** 2 + 8))
    s2 = (1 / den) * (1.5 * c3 * (2 * a22 * (k ** 2 - 2) + a24 * (k ** 2 + 2) + 2 * k * b22 + 5 * d21)
                      + 0.375 * c4 * (12 - k ** 2))
    a1 = -1.5 * c3 * (2 * a21 + a23 + 5 * d21) - 0.375 * c4 * (12 - k ** 2)
    a2 = 1.5 * c3 * (a24 - 2 * a22) + 1.125 * c4
    l1 = a1 + 2 * lam ** 2 * s1
    l2 = a2 + 2 * lam ** 2 * s2
    Ax = np.sqrt((-delta - l2 * Az ** 2) / l1)
    # tau1 = 0: cos = 1, sin = 0
    x = a21 * Ax ** 2 + a22 * Az ** 2 - Ax + (a23 * Ax ** 2 - a24 * Az ** 2) + (a31 * Ax ** 3 - a32 * Ax * Az ** 2)
    z = deltan * Az + deltan * d21 * Ax * Az * (1.0 - 3.0) + deltan * (d32 * Az * Ax ** 2 - d31 * Az ** 3)
    ydot = lam * (k * Ax + 2 * (b21 * Ax ** 2 - b22 * Az ** 2) + 3 * (b31 * Ax ** 3 - b32 * Ax * Az ** 2))
    won = 1.0 if point == 1 else -1.0
    primary = 1.0 - mu
    out = np.zeros((Az.size, 6))
    out[:, 0] = primary + g * (-won + x)
    out[:, 2] = g * z
    out[:, 4] = g * ydot
    return out
