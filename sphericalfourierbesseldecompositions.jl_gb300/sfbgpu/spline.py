"""Cubic spline tables for the g_nl(r) radial basis (host side).

The reference caches every g_nl(r) as a ``Spline1D{3}`` (reference
``src/Splines.jl:20-28``) and evaluates that spline once per galaxy inside
``cat2amln`` (``src/cat2anlm.jl:95-103``).  The GPU plan receives the same
knots ``x``, values ``y`` and second derivatives ``ypp`` that a Julia caller
would pass, so the construction below keeps the reference's end conditions
and forward/backward sweep (``src/Splines.jl:179-182,206-271``).

Construction is vectorised over many splines of different lengths at once:
one sweep row ``i`` is advanced for every spline simultaneously, and each
spline's own last interior row is selected through a mask.  The arithmetic of
each individual spline is the reference's, step for step.
"""

import numpy as np

__all__ = ["build_ypp_batched", "build_ypp", "eval_spline"]


def build_ypp(x, y):
    """Second derivatives of one cubic spline (reference src/Splines.jl:206-271)."""
    ypp, = build_ypp_batched([np.asarray(x, float)], [np.asarray(y, float)])
    return ypp


def build_ypp_batched(xs, ys):
    """Second-derivative tables for a list of splines (each needs >= 4 knots).

    Returns a list of arrays, one per spline.  Rows are 0-based here: the
    reference's 1-based row ``i`` is row ``i-1``.  Work arrays are laid out
    (row, spline) so that one sweep step touches contiguous memory.
    """
    S = len(xs)
    if S == 0:
        return []
    N = np.array([len(x) for x in xs], dtype=np.int64)
    if np.any(N < 4):
        raise ValueError("cubic spline needs at least 4 knots")
    Nmax = int(N.max())
    X = np.empty((Nmax, S))
    Y = np.empty((Nmax, S))
    for s in range(S):
        n = N[s]
        X[:n, s] = xs[s]
        Y[:n, s] = ys[s]
        if n < Nmax:
            # padding rows continue the last knot spacing so they stay finite
            h = xs[s][-1] - xs[s][-2]
            X[n:, s] = xs[s][-1] + h * np.arange(1, Nmax - n + 1)
            Y[n:, s] = ys[s][-1]
    cols = np.arange(S)
    last = N - 1                                  # row of the reference's x[N]

    # End conditions from three-point parabola slopes (Splines.jl:179-182,232-240).
    x1, x2, x3 = X[0], X[1], X[2]
    y1, y2, y3 = Y[0], Y[1], Y[2]
    yp1 = ((y3 - y1) * (x2 - x1) ** 2 - (y2 - y1) * (x3 - x1) ** 2) / (
        (x3 - x1) * (x2 - x3) * (x2 - x1))
    A2adj = 3 * yp1 - 3 * (y2 - y1) / (x2 - x1)
    a22adj = -(x2 - x1) / 2
    xN, xN1, xN2 = X[last, cols], X[last - 1, cols], X[last - 2, cols]
    yN, yN1, yN2 = Y[last, cols], Y[last - 1, cols], Y[last - 2, cols]
    ypN = ((yN2 - yN) * (xN1 - xN) ** 2 - (yN1 - yN) * (xN2 - xN) ** 2) / (
        (xN2 - xN) * (xN1 - xN2) * (xN1 - xN))
    ANadj = 3 * (yN - yN1) / (xN - xN1) - 3 * ypN
    aNNadj = -(xN - xN1) / 2

    def Ai(i):
        return (6 * (Y[i + 1] - Y[i]) / (X[i + 1] - X[i])
                - 6 * (Y[i] - Y[i - 1]) / (X[i] - X[i - 1]))

    betainv = np.zeros((Nmax, S))
    u = np.zeros((Nmax, S))
    # forward substitution (Splines.jl:244-254)
    betainv[1] = 1 / (2 * (X[2] - X[0]) + a22adj)
    u[1] = Ai(1) + A2adj
    for i in range(2, Nmax - 1):
        t = (X[i] - X[i - 1]) * betainv[i - 1]
        is_last = (i == last - 1)
        # The last interior row adds aNNadj / ANadj before the elimination
        # term is subtracted, in the reference's operation order.
        denom = np.where(is_last,
                         2 * (X[i + 1] - X[i - 1]) + aNNadj - (X[i] - X[i - 1]) * t,
                         2 * (X[i + 1] - X[i - 1]) - (X[i] - X[i - 1]) * t)
        betainv[i] = 1 / denom
        a_i = Ai(i)
        u[i] = np.where(is_last, a_i + ANadj - t * u[i - 1], a_i - t * u[i - 1])
    # backward substitution (Splines.jl:257-263)
    ypp = np.zeros((Nmax, S))
    ypp[last - 1, cols] = betainv[last - 1, cols] * u[last - 1, cols]
    for i in range(Nmax - 3, 0, -1):
        active = i <= last - 2
        val = betainv[i] * (u[i] - (X[i + 1] - X[i]) * ypp[i + 1])
        ypp[i] = np.where(active, val, ypp[i])
    ypp[0] = (a22adj * ypp[1] - A2adj) / (x2 - x1)
    ypp[last, cols] = (aNNadj * ypp[last - 1, cols] - ANadj) / (xN - xN1)
    return [ypp[:N[s], s].copy() for s in range(S)]


def eval_spline(x, y, ypp, r):
    """Evaluate a cubic spline with boundary extrapolation at points ``r``.

    Same piece selection (largest knot <= r), cubic coefficients and Horner
    order as the reference (src/Splines.jl:64-101,327-357); outside
    [x[0], x[-1]] the end value is returned (extrapolation=boundary).
    """
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    ypp = np.asarray(ypp, float)
    r = np.asarray(r, float)
    N = len(x)
    i = np.searchsorted(x, r, side="right") - 1          # 0-based piece start
    below = r < x[0]
    above = r > x[-1]
    i = np.clip(i, 0, N - 2)
    x0 = x[i]
    h = x[i + 1] - x0
    t = (r - x0) / h
    h2 = h * h
    b = h2 * ypp[i] / 2
    a = h2 * (ypp[i + 1] - ypp[i]) / 6
    d = y[i]
    c = y[i + 1] - a - b - d
    val = d + t * (c + t * (b + t * a))
    val = np.where(below, y[0], val)
    val = np.where(above, y[-1], val)
    return val
