"""The rays driver's distance statistics (src/rays.cpp:280-455), host side.

For each central trajectory of the bundles (``rays_propagate``) the driver
forms a pair (x, y): x the interpolation parameter, y the statistic; the
pairs are re-interpolated on a grid taken from the FLRW reference bundle
(every statmod-th point, nstat points in all), and the mean and standard
deviation over rays are reduced over the ranks.  This module restates that
arithmetic in float64 numpy, in the reference's order, with the reduction
through ``torch.distributed`` when a process group is given (the one
collective of the rays path: an all-reduce of three short vectors).

The reference's case mapping is kept as it is: with interpolation "a" the
x value of the rays is their conformal time t and with "t" it is 1/a - 1
(rays.cpp:297-318, 331-345), while the reference grid follows the same
mapping, so the two stay consistent.
"""
from __future__ import annotations

import numpy as np

STATISTICS = ("distance", "distance2", "homogeneous", "inhomogeneous", "invdistance", "invdistance2")
# trajectory file columns
_T, _A, _X, _RED, _DIST, _LAMBDA = 2, 1, 3, 19, 22, 26

_INTERP_CASE = {"redshift": 0, "a": 1, "t": 2, "r": 3, "lambda": 4}
_STAT_CASE = {name: i for i, name in enumerate(STATISTICS)}


def _x(traj, case):
    if case == 1:
        return traj[:, _T].copy()
    if case == 2:
        return 1.0 / traj[:, _A] - 1.0
    if case == 3:
        d = traj[:, _X:_X + 3] - traj[0, _X:_X + 3]
        return np.sqrt(d[:, 0] ** 2 + d[:, 1] ** 2 + d[:, 2] ** 2)
    if case == 4:
        return traj[:, _LAMBDA].copy()
    return traj[:, _RED].copy()


def _y(traj, case, invlength):
    d = traj[:, _DIST] * invlength
    if case == 1:
        return d * d
    if case == 2:
        return traj[0, _A] / traj[:, _A] - 1.0
    if case == 3:
        return traj[:, _RED].copy()
    if case == 4:
        return 1.0 / d
    if case == 5:
        return 1.0 / (d * d)
    return d


def interpolate(x0, x, y):
    """Utility::interpolate (utility.h:441-449) at every x0: upper_bound, then
    the bracketing segment, clamped to the end segments."""
    x0 = np.asarray(x0, dtype=np.float64)
    n = min(len(x), len(y))
    if n == 0:
        return np.zeros_like(x0)
    if n == 1:
        return np.full_like(x0, y[0])
    i = np.searchsorted(x[:n], x0, side="right")
    i = i + ((i <= 0).astype(np.int64) - (i >= n).astype(np.int64))
    return y[i - 1] + ((y[i] - y[i - 1]) * (x0 - x[i - 1]) / (x[i] - x[i - 1]))


def _allreduce(dist, values):
    if dist is None:
        return values
    import torch
    t = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64))
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t)
    return t.cpu().numpy()


def statistics(central, reference, interpolation="redshift", statistic="distance", amin=0.0, nstat=100,
               invlength=1.0, dist=None):
    """central: the central trajectories (m_i x 29) of this rank's bundles, the
    rejected ones (size 0) included or not; reference: the FLRW reference
    bundle's central trajectory (m x 29).  Returns a dict with the grid
    (z: redshift, y: the statistic along the reference), this rank's mean and
    std, the reduced mean and std and the counts (rays.cpp:300-434)."""
    icase = _INTERP_CASE.get(interpolation, 0)
    scase = _STAT_CASE.get(statistic, 0)
    statx, staty = [], []
    for traj in central:
        traj = np.asarray(traj, dtype=np.float64)
        if traj.shape[0] == 0:
            continue
        statx.append(_x(traj, icase))
        staty.append(_y(traj, scase, invlength))
    ref = np.asarray(reference, dtype=np.float64)
    if np.isfinite(amin) and abs(amin) >= np.finfo(np.float64).tiny:   # std::isnormal(amin)
        ref = ref[~(ref[:, _A] < amin)]
    statmod = max(1, ref.shape[0] // max(int(nstat), 1))
    keep = np.arange(ref.shape[0]) % statmod == 0
    refx = _x(ref, icase)[keep] if ref.shape[0] else np.zeros(0)
    refy = _y(ref, scase, invlength)[keep] if ref.shape[0] else np.zeros(0)
    refz = ref[keep, _RED] if ref.shape[0] else np.zeros(0)
    n = refx.shape[0]
    ys = np.array([interpolate(refx, x, y) for x, y in zip(statx, staty)]).reshape(len(staty), n)
    size = ys.shape[0]
    gsize = int(round(_allreduce(dist, np.array([float(size)]))[0]))
    s = ys.sum(axis=0) if size else np.zeros(n)
    gmean = _allreduce(dist, s) / float(gsize) if gsize else np.full(n, np.nan)
    mean = s / float(size) if size else np.full(n, np.nan)
    gvar = _allreduce(dist, ((ys - gmean) ** 2).sum(axis=0) if size else np.zeros(n))
    var = ((ys - mean) ** 2).sum(axis=0) if size else np.zeros(n)
    wrap = 1 << 32    # the counts are unsigned in the reference
    with np.errstate(divide="ignore", invalid="ignore"):
        std = np.sqrt(var / float((size - 1) % wrap))
        gstd = np.sqrt(gvar / float((gsize - 1) % wrap))
    return dict(z=refz, y=refy, x=refx, mean=mean, std=std, gmean=gmean, gstd=gstd, count=size, gcount=gsize)


def statistics_text(z, y, mean, std, count) -> str:
    """Output::save(stream, x, y, ymean, ystd, digits, count) (output.h:227-243):
    a '# count' line, then 'x y mean std' at 17 significant digits."""
    lines = ["# %d" % int(count)]
    for v in zip(z, y, mean, std):
        lines.append(" ".join("%.17g" % float(q) for q in v))
    return "".join(l + "\n" for l in lines)
