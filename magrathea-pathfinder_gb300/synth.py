"""Seeded synthetic inputs for the photon-propagation path.

The reference reads RAMSES cell dumps; no such data ship here, so this module
generates octrees with the shapes and value distributions of the standard
workloads and writes them in the reference's own on-disk cone format
(raw 48-byte records sorted by key, ``src/input.h:1275-1313``):

====  =====================================================================
byte  field (``Gravity<float,3>`` in a ``std::pair`` with a 128-bit key)
====  =====================================================================
0-15  key, ``unsigned __int128`` little-endian (low 64 bits first)
16    dphidt (f32)       20  a (f32)
24    dphidx (f32)       28  dphidy (f32)      32  dphidz (f32)
36    phi (f32)          40  rho (f32)         44  padding
====  =====================================================================

Keys follow ``SimpleHyperOctreeIndex<__uint128_t,3>``
(``src/magrathea/simplehyperoctreeindex.h:1165-1189``): level ``L`` uses the
top ``4L`` bits, one nibble per level from the most significant end, each
nibble ``1zyx`` (marker bit, then the z, y, x bits of the cell coordinate,
most significant coordinate bit first).  The integer coordinate along each
axis is ``trunc((1/E) * 2**L * (x - (-E/2)))`` with the octree extent
``E = 4`` (EXTENT in the reference Makefile), evaluated in float64 in exactly
that order, then masked to ``L`` bits.

Fields are in SI units as the reference stores them after
``Input::sistemize`` (``src/input.h:368-379``): phi in m^2/s^2, dphidx..z the
gradient with respect to comoving metres, dphidt in m^2/s^3.  Positions are
in box units with the observer at the origin and, as for the reference's
narrow cones after rotation, the cone axis along +x.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

EXTENT = 4
C_LIGHT = 299792458.0
MPC = 3.08568e22
G_NEWTON = 6.674e-11
MSUN = 1.98847e30

RECORD = np.dtype([
    ("lo", "<u8"), ("hi", "<u8"),
    ("dphidt", "<f4"), ("a", "<f4"),
    ("dphidx", "<f4"), ("dphidy", "<f4"), ("dphidz", "<f4"),
    ("phi", "<f4"), ("rho", "<f4"), ("pad", "<u4"),
])
assert RECORD.itemsize == 48


# --------------------------------------------------------------------------
# keys
# --------------------------------------------------------------------------
def coords(level: int, pos: np.ndarray) -> np.ndarray:
    """Integer cell coordinates at ``level`` of positions ``pos`` [..., 3].

    Same float64 operation order as ``SimpleHyperOctreeIndex::compute``:
    ``(den/num) * 2**L`` first (exact), times ``(x - ref)``, truncated.
    Negative values (positions below the extent) saturate to 0 here; the
    reference's conversion of a negative double to unsigned is undefined
    there, and valid inputs never reach it.
    """
    pos = np.asarray(pos, dtype=np.float64)
    scale = (1.0 / EXTENT) * float(2 ** level)
    v = scale * (pos - (-EXTENT / 2.0))
    v = np.where(v > 0.0, v, 0.0)
    c = np.floor(v).astype(np.uint64)
    mask = np.uint64((1 << level) - 1) if level < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    return c & mask


def key_from_coords(level: int, c: np.ndarray):
    """(hi, lo) uint64 halves of the level-``level`` key of integer coords."""
    c = np.asarray(c, dtype=np.uint64)
    hi = np.zeros(c.shape[:-1], dtype=np.uint64)
    lo = np.zeros(c.shape[:-1], dtype=np.uint64)
    for k in range(1, level + 1):
        b = np.uint64(level - k)
        nib = (np.uint64(8)
               | (((c[..., 2] >> b) & np.uint64(1)) << np.uint64(2))
               | (((c[..., 1] >> b) & np.uint64(1)) << np.uint64(1))
               | ((c[..., 0] >> b) & np.uint64(1)))
        if k <= 16:
            hi |= nib << np.uint64(64 - 4 * k)
        else:
            lo |= nib << np.uint64(128 - 4 * k)
    return hi, lo


def compute_key(level: int, pos: np.ndarray):
    """``SimpleHyperOctreeIndex::compute(level, x, y, z)`` as (hi, lo)."""
    return key_from_coords(level, coords(level, pos))


def cipher_key(pos: np.ndarray):
    """``SimpleHyperOctreeIndex::cipher(x, y, z)``: the level-32 key."""
    return compute_key(32, pos)


def key_level(hi: np.ndarray, lo: np.ndarray) -> np.ndarray:
    """Level = number of leading nibbles whose marker bit is set."""
    hi = np.asarray(hi, dtype=np.uint64)
    lo = np.asarray(lo, dtype=np.uint64)
    lev = np.zeros(hi.shape, dtype=np.int64)
    for k in range(1, 33):
        word = hi if k <= 16 else lo
        sh = np.uint64(64 - 4 * k) if k <= 16 else np.uint64(128 - 4 * k)
        bit = ((word >> (sh + np.uint64(3))) & np.uint64(1)).astype(bool)
        lev = np.where(bit, k, lev)
    return lev


def key_coords(hi, lo, level):
    """Inverse of key_from_coords for keys of one known level."""
    hi = np.asarray(hi, dtype=np.uint64)
    lo = np.asarray(lo, dtype=np.uint64)
    c = np.zeros(hi.shape + (3,), dtype=np.uint64)
    for k in range(1, level + 1):
        word = hi if k <= 16 else lo
        sh = np.uint64(64 - 4 * k) if k <= 16 else np.uint64(128 - 4 * k)
        nib = (word >> sh) & np.uint64(15)
        b = np.uint64(level - k)
        for d in range(3):
            c[..., d] |= ((nib >> np.uint64(d)) & np.uint64(1)) << b
    return c


def cell_center(level: int, c: np.ndarray) -> np.ndarray:
    """Cell centre, ``ref + E * (2c+1) / 2**(L+1)`` (exact in float64)."""
    c = np.asarray(c, dtype=np.float64)
    return -EXTENT / 2.0 + EXTENT * ((2.0 * c + 1.0) / float(2 ** (level + 1)))


# --------------------------------------------------------------------------
# cosmology
# --------------------------------------------------------------------------
@dataclass
class Cosmology:
    h: float = 0.68
    omega_m: float = 0.31

    @property
    def H0(self) -> float:  # 1/s
        return self.h * 1e5 / MPC

    def E(self, a):
        a = np.asarray(a, dtype=np.float64)
        return np.sqrt(self.omega_m / a ** 3 + 1.0 - self.omega_m)

    def chi_of_z(self, z):
        """Comoving distance in Mpc/h (flat LCDM)."""
        z = np.atleast_1d(np.asarray(z, dtype=np.float64))
        zz = np.linspace(0.0, max(float(z.max()), 1e-6) * 1.001 + 1e-3, 40001)
        Ez = np.sqrt(self.omega_m * (1 + zz) ** 3 + 1 - self.omega_m)
        dc = np.concatenate([[0.0], np.cumsum(0.5 * (1 / Ez[1:] + 1 / Ez[:-1]) * np.diff(zz))])
        return np.interp(z, zz, dc) * (C_LIGHT / 1e5)

    def z_of_chi(self, chi):
        zz = np.linspace(0.0, 12.0, 120001)
        dc = self.chi_of_z(zz)
        return np.interp(np.asarray(chi, dtype=np.float64), dc, zz)

    def growth_rate(self, a):
        a = np.asarray(a, dtype=np.float64)
        om_a = self.omega_m / a ** 3 / self.E(a) ** 2
        return om_a ** 0.55

    def evolution_table(self, n: int = 2000, amin: float = 1e-3):
        """RAMSES-style evolution file columns (a, a^2 E(a), 0, 0, t_proper*H0);
        ``Input::acquire`` reads columns 0, 1 and 4 (``src/input.h:1167-1170``)."""
        aa = np.linspace(amin, 1.0, n)
        Ea = self.E(aa)
        integrand = 1.0 / (aa * Ea)
        tp = np.concatenate([[0.0], np.cumsum(np.diff(aa) * 0.5 * (integrand[1:] + integrand[:-1]))])
        tp -= tp[-1]
        return np.column_stack([aa, aa ** 2 * Ea, np.zeros_like(aa), np.zeros_like(aa), tp])

    def conformal_table(self, n: int = 4000, amin: float = 0.05):
        """Table in the layout the integrator consumes: conformal time t in
        seconds, zero at the observer and increasing into the past, a(t),
        da/dt (negative) and d2a/dt2, rows ordered by increasing t."""
        aa = np.linspace(1.0, amin, n)
        H = self.H0 * self.E(aa)
        dtda = -1.0 / (aa * aa * H)                    # dt_conf/da along decreasing a
        t = np.concatenate([[0.0], np.cumsum(0.5 * (dtda[1:] + dtda[:-1]) * np.diff(aa))])
        dadt = -aa * aa * H
        # d2a/dt2 = d(dadt)/da * dadt
        d_dadt_da = -(2 * aa * H + aa * aa * self.H0 * np.gradient(self.E(aa), aa))
        d2adt2 = d_dadt_da * dadt
        return t, aa, dadt, d2adt2


def write_param_files(directory: str, cosmo: Cosmology, lbox: float, phi_deg: int = 20,
                      theta_deg: float = 20.0, half_y: float = 2.5, half_z: float = 2.5):
    """Cosmology inputs in the reference's formats: ``param.txt`` (h, Omega_m),
    ``evol.dat`` and a ``boxlen<L>_…/`` cell directory with
    ``info_narrow_cone.txt``.  Returns (celldir, paramfile, evolfile)."""
    os.makedirs(directory, exist_ok=True)
    paramfile = os.path.join(directory, "param.txt")
    evolfile = os.path.join(directory, "evol.dat")
    celldir = os.path.join(directory, "boxlen%g_synthetic" % lbox, "cells") + os.sep
    os.makedirs(celldir, exist_ok=True)
    with open(paramfile, "w") as f:
        f.write("h=%.8f\nOmega_m=%.8f\n" % (cosmo.h, cosmo.omega_m))
    np.savetxt(evolfile, cosmo.evolution_table(), fmt="%.12e")
    with open(os.path.join(celldir, "info_narrow_cone.txt"), "w") as f:
        f.write("phi = %d\ntheta = %g\nthetay = %g\nthetaz = %g\n" % (phi_deg, theta_deg, half_y, half_z))
    return celldir, paramfile, evolfile


# --------------------------------------------------------------------------
# fields
# --------------------------------------------------------------------------
def gaussian_field(n: int, seed: int, kc_over_2pi: float = 16.0) -> np.ndarray:
    """Periodic Gaussian random field with P(k) ~ k^-3 exp(-(k/kc)^2),
    k in units of 2*pi/box, unit rms."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n) * n * 2 * np.pi
    kx, ky, kz = np.meshgrid(k, k, np.fft.rfftfreq(n) * n * 2 * np.pi, indexing="ij")
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    kk[0, 0, 0] = 1.0
    kc = kc_over_2pi * 2 * np.pi
    amp = np.sqrt(kk ** -3.0 * np.exp(-(kk / kc) ** 2))
    amp[0, 0, 0] = 0.0
    noise = np.fft.rfftn(rng.standard_normal((n, n, n)))
    f = np.fft.irfftn(noise * amp, s=(n, n, n), axes=(0, 1, 2))
    return f / f.std()


def _trilinear_periodic(grid: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Periodic trilinear interpolation; u in grid-index units (cell centres
    at integers)."""
    n = grid.shape[0]
    f = np.floor(u)
    w = u - f
    i0 = f.astype(np.int64) % n
    i1 = (i0 + 1) % n
    out = np.zeros(u.shape[0], dtype=np.float64)
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1 - w[:, 0]
        ix = i1[:, 0] if dx else i0[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1 - w[:, 1]
            iy = i1[:, 1] if dy else i0[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1 - w[:, 2]
                iz = i1[:, 2] if dz else i0[:, 2]
                out += wx * wy * wz * grid[ix, iy, iz]
    return out


@dataclass
class OctreeSpec:
    """A synthetic cone octree.

    base_level   octree level of the base grid (file level + log2(EXTENT))
    box_cells    cells per box side of the periodic base field (2**file_level)
    lbox         box length in Mpc/h
    half_y/z     cone half-angles (degrees) about +x
    chi_max      comoving depth to cover, Mpc/h
    margin       extra cells kept around the cone and the observer
    halos        number of NFW halos (0 = uniform grid)
    max_level    finest octree level inside halos
    """
    base_level: int = 8
    box_cells: int = 64
    lbox: float = 2048.0
    half_y: float = 2.5
    half_z: float = 2.5
    chi_max: float = 1400.0
    margin: int = 3
    seed: int = 42
    phi_rms_c2: float = 1e-5
    halos: int = 0
    max_level: int = 8
    mass_min: float = 1e12
    mass_max: float = 1e15
    concentration: float = 5.0
    refine_cells: float = 2.5
    cosmo: Cosmology = field(default_factory=Cosmology)
    axis_deg: tuple = None   # (phi, theta) of the cone axis (narrow_cone_axis); None: +x

    def frame(self) -> np.ndarray:
        """3x3 rotation whose columns are the cone frame's axes in octree
        coordinates (column 0: the cone axis)."""
        return np.eye(3) if self.axis_deg is None else cone_frame(*self.axis_deg)


def narrow_cone_axis(phi_deg: float, theta_deg: float) -> np.ndarray:
    """Axis of a narrow cone of the reference's cone parameters (phi, theta):
    (cos(theta) cos(phi), -sin(phi), cos(phi) sin(theta)) (src/miscellaneous.h:315-325,
    src/input.h:1030-1040)."""
    ph, th = math.radians(phi_deg), math.radians(theta_deg)
    return np.array([math.cos(th) * math.cos(ph), -math.sin(ph), math.cos(ph) * math.sin(th)])


def cone_frame(phi_deg: float, theta_deg: float) -> np.ndarray:
    """Right-handed orthonormal frame with the narrow cone's axis as its
    first column; the second column is horizontal (no z component)."""
    n = narrow_cone_axis(phi_deg, theta_deg)
    ey = np.cross([0.0, 0.0, 1.0], n)
    ey /= np.linalg.norm(ey)
    ez = np.cross(n, ey)
    return np.stack([n, ey, ez], axis=1)


def uniform_grid_cone(z_max: float = 0.5, axis_deg=(20.0, 20.0), lbox: float = 2048.0, half_deg: float = 2.5,
                      seed: int = 42) -> OctreeSpec:
    """The 64^3 periodic field at file level 6 (octree level 8, no refinement)
    over a 2 half_deg square cone along the narrow cone axis (phi, theta) =
    axis_deg, deep enough for rays to z_max."""
    cosmo = Cosmology()
    chi = float(cosmo.chi_of_z(z_max)[0])
    return OctreeSpec(base_level=8, box_cells=64, lbox=lbox, half_y=half_deg, half_z=half_deg, chi_max=chi * 1.02,
                      halos=0, max_level=8, seed=seed, axis_deg=tuple(axis_deg))


def _cone_mask(centers: np.ndarray, spec: OctreeSpec, cell: float) -> np.ndarray:
    local = centers @ spec.frame()          # coordinates in the cone frame
    x, y, z = local[:, 0], local[:, 1], local[:, 2]
    pad = spec.margin * cell
    ty = math.tan(math.radians(spec.half_y))
    tz = math.tan(math.radians(spec.half_z))
    xmax = spec.chi_max / spec.lbox + pad
    in_cone = (x > -pad) & (x < xmax) & (np.abs(y) <= np.maximum(x, 0) * ty + pad) & \
              (np.abs(z) <= np.maximum(x, 0) * tz + pad)
    near_obs = np.max(np.abs(centers), axis=1) <= pad + cell
    return in_cone | near_obs


def _base_cells(spec: OctreeSpec) -> np.ndarray:
    """Integer coords at base_level of the cells covering the cone."""
    L = spec.base_level
    cell = EXTENT / 2.0 ** L
    pad = spec.margin * cell
    ty = math.tan(math.radians(spec.half_y))
    tz = math.tan(math.radians(spec.half_z))
    xmax = spec.chi_max / spec.lbox + pad
    # bounding box of the cone frame's box around the cone, in octree coordinates
    corners = np.array([[x, y, z] for x in (-pad - cell, xmax + cell) for y in (-(xmax * ty + pad), xmax * ty + pad + cell)
                        for z in (-(xmax * tz + pad), xmax * tz + pad + cell)]) @ spec.frame().T
    lo = coords(L, np.maximum(corners.min(axis=0) - cell, -EXTENT / 2.0))
    hi = coords(L, np.minimum(corners.max(axis=0) + cell, EXTENT / 2.0 - 1e-12))
    out = []
    ys = np.arange(int(lo[1]), int(hi[1]) + 1, dtype=np.int64)
    zs = np.arange(int(lo[2]), int(hi[2]) + 1, dtype=np.int64)
    Y, Z = np.meshgrid(ys, zs, indexing="ij")
    for ix in range(int(lo[0]), int(hi[0]) + 1):
        c = np.stack([np.full(Y.size, ix, dtype=np.int64), Y.ravel(), Z.ravel()], axis=1)
        m = _cone_mask(cell_center(L, c), spec, cell)
        if m.any():
            out.append(c[m])
    return np.concatenate(out).astype(np.uint64)


def _nfw_halos(spec: OctreeSpec, rng: np.random.Generator):
    """Halo centres (box units), r_s and 4 pi G rho_s r_s^3 (SI) and cutoff."""
    cosmo = spec.cosmo
    n = spec.halos
    ty = math.tan(math.radians(spec.half_y))
    tz = math.tan(math.radians(spec.half_z))
    xmax = spec.chi_max / spec.lbox
    # uniform in the cone volume: x ~ x^2
    x = xmax * rng.random(n) ** (1.0 / 3.0)
    x = np.maximum(x, 0.05 * xmax)
    y = (2 * rng.random(n) - 1) * x * ty
    z = (2 * rng.random(n) - 1) * x * tz
    centres = np.stack([x, y, z], axis=1) @ spec.frame().T
    mass = np.exp(rng.uniform(math.log(spec.mass_min), math.log(spec.mass_max), n))  # Msun/h
    rho_c = 2.775e11  # h^2 Msun / Mpc^3
    r200 = (3 * mass / (4 * math.pi * 200 * rho_c)) ** (1.0 / 3.0)  # Mpc/h comoving
    rs = r200 / spec.concentration
    cc = spec.concentration
    mu = math.log(1 + cc) - cc / (1 + cc)
    # 4 pi G rho_s r_s^3 = G M / mu  (SI, with M in kg)
    gm = G_NEWTON * mass / cosmo.h * MSUN / mu
    return centres, rs, r200, gm


def _nfw_phi_grad(d_m: np.ndarray, rs_m: float, gm: float, rc_m: float):
    """C1-truncated NFW potential and radial derivative (SI, metres)."""
    r = np.maximum(d_m, 1e-3 * rs_m)

    def phi(r):
        return -gm * np.log1p(r / rs_m) / r

    def dphi(r):
        return gm * (np.log1p(r / rs_m) / r ** 2 - 1.0 / (r * (rs_m + r)))

    p = phi(r) - phi(rc_m) - (r - rc_m) * dphi(rc_m)
    g = dphi(r) - dphi(rc_m)
    inside = d_m < rc_m
    return np.where(inside, p, 0.0), np.where(inside, g, 0.0)


def make_octree(spec: OctreeSpec, verbose: bool = False) -> np.ndarray:
    """Build the synthetic cone octree; returns sorted RECORD array."""
    rng = np.random.default_rng(spec.seed)
    cosmo = spec.cosmo
    length_m = spec.lbox * MPC / cosmo.h
    n = spec.box_cells
    grf = gaussian_field(n, spec.seed, 16.0)
    phi_amp = spec.phi_rms_c2 * C_LIGHT ** 2
    phi_grid = grf * phi_amp
    dx_m = length_m / n
    grads = [(np.roll(phi_grid, -1, d) - np.roll(phi_grid, 1, d)) / (2 * dx_m) for d in range(3)]
    lap = sum(np.roll(phi_grid, -1, d) + np.roll(phi_grid, 1, d) for d in range(3)) - 6 * phi_grid
    rho_grid = 1.0 + 0.3 * lap / lap.std()

    levels = {spec.base_level: _base_cells(spec)}
    halos = None
    if spec.halos > 0:
        halos = _nfw_halos(spec, rng)
        hc, rs, r200, gm = halos
        L = spec.base_level
        while L < spec.max_level:
            cell = EXTENT / 2.0 ** L
            cur = levels[L]
            ctr = cell_center(L, cur)
            refine = np.zeros(cur.shape[0], dtype=bool)
            # bucket halos by base-level cell to limit the search
            radius = r200 / spec.lbox + spec.refine_cells * cell
            order = np.argsort(ctr[:, 0])
            xs = ctr[order, 0]
            for k in range(hc.shape[0]):
                lo_i = np.searchsorted(xs, hc[k, 0] - radius[k])
                hi_i = np.searchsorted(xs, hc[k, 0] + radius[k])
                if hi_i <= lo_i:
                    continue
                idx = order[lo_i:hi_i]
                d = np.linalg.norm(ctr[idx] - hc[k], axis=1)
                refine[idx[d < radius[k]]] = True
            parents = cur[refine]
            if parents.shape[0] == 0:
                break
            kids = (parents[:, None, :] * np.uint64(2) +
                    np.array([[(s >> 0) & 1, (s >> 1) & 1, (s >> 2) & 1] for s in range(8)], dtype=np.uint64)[None])
            levels[L + 1] = kids.reshape(-1, 3)
            L += 1

    recs = []
    for L, c in sorted(levels.items()):
        ctr = cell_center(L, c)
        # base-field index coordinates: the observer sits on a box corner
        u = (ctr * n)  # box units -> base cells; cell centres at k+0.5
        u = u - 0.5
        phi = _trilinear_periodic(phi_grid, u)
        g = np.stack([_trilinear_periodic(gr, u) for gr in grads], axis=1)
        rho = _trilinear_periodic(rho_grid, u)
        if halos is not None:
            hc, rs, r200, gm = halos
            rcut = 4.0 * r200 / spec.lbox
            order = np.argsort(ctr[:, 0])
            xs = ctr[order, 0]
            for k in range(hc.shape[0]):
                lo_i = np.searchsorted(xs, hc[k, 0] - rcut[k])
                hi_i = np.searchsorted(xs, hc[k, 0] + rcut[k])
                if hi_i <= lo_i:
                    continue
                idx = order[lo_i:hi_i]
                dv = (ctr[idx] - hc[k]) * length_m
                d = np.linalg.norm(dv, axis=1)
                sel = d < rcut[k] * length_m
                if not sel.any():
                    continue
                idx, dv, d = idx[sel], dv[sel], d[sel]
                p, gr = _nfw_phi_grad(d, rs[k] * MPC / cosmo.h, gm[k], rcut[k] * length_m)
                phi[idx] += p
                g[idx] += (gr / np.maximum(d, 1e-30))[:, None] * dv
                rho[idx] += -p / phi_amp
        chi = np.linalg.norm(ctr, axis=1) * spec.lbox
        a = 1.0 / (1.0 + cosmo.z_of_chi(chi))
        aH = a * cosmo.H0 * cosmo.E(a)
        dphidt = phi * (1.0 - cosmo.growth_rate(a)) * aH
        hi, lo = key_from_coords(L, c)
        r = np.zeros(c.shape[0], dtype=RECORD)
        r["hi"], r["lo"] = hi, lo
        r["dphidt"] = dphidt
        r["a"] = a
        r["dphidx"], r["dphidy"], r["dphidz"] = g[:, 0], g[:, 1], g[:, 2]
        r["phi"] = phi
        r["rho"] = rho
        recs.append(r)
        if verbose:
            print("level %d: %d cells" % (L, c.shape[0]))
    out = np.concatenate(recs)
    order = np.lexsort((out["lo"], out["hi"]))
    return out[order]


def cells_ramses(records: np.ndarray, spec: OctreeSpec) -> np.ndarray:
    """The cells of an octree as the 10-column ASCII rows create_octree reads
    (level, x, y, z, rho, phi, force x y z, a; input.h:1023-1025): RAMSES file
    level (octree level - log2 EXTENT), centre in octree units, and phi and
    force in RAMSES units -- the inverse of Input::sistemize (input.h:368-379):
    phi_SI = phi (l/t)^2, dphidx_SI = force (l/t^2)(-a), l = a lbox mpc / h,
    t = a^2 mpc / (h 1e5).  dphidt is not an input (create_octree derives it)."""
    lev = key_level(records["hi"], records["lo"]).astype(np.int64)
    out = np.zeros((records.shape[0], 10))
    for L in np.unique(lev):
        m = lev == L
        out[m, 1:4] = cell_center(int(L), key_coords(records["hi"][m], records["lo"][m], int(L)))
    out[:, 0] = lev - int(np.log2(EXTENT))
    a = records["a"].astype(np.float64)
    h = spec.cosmo.h
    t = a * a * MPC / (h * 1e5)
    l = a * spec.lbox * MPC / h
    out[:, 4] = records["rho"]
    out[:, 5] = records["phi"] * (t / l) ** 2
    for q, name in enumerate(("dphidx", "dphidy", "dphidz")):
        out[:, 6 + q] = records[name] / ((l / (t * t)) * (-a))
    out[:, 9] = a
    return out


def write_cells(path: str, rows: np.ndarray) -> None:
    """ASCII cell file: integer level, then 9 values at float precision."""
    with open(path, "w") as f:
        for r in rows:
            f.write("%d %s\n" % (int(r[0]), " ".join("%.9g" % v for v in r[1:])))


def write_bin(path: str, records: np.ndarray) -> None:
    records.astype(RECORD, copy=False).tofile(path)


def read_bin(path: str) -> np.ndarray:
    return np.fromfile(path, dtype=RECORD)


def photon_grid(n_side: int, half_y_deg: float, half_z_deg: float, frame=None) -> np.ndarray:
    """Launch records (x0 y0 z0 x1 y1 z1) for an n_side x n_side grid of
    directions filling the square cone about +x, in the reference's
    narrow-cone angles (|phi| < half_y, |theta - pi/2| < half_z); with
    `frame` (OctreeSpec.frame()), about that frame's first axis."""
    t = (np.arange(n_side) + 0.5) / n_side * 2.0 - 1.0
    ph = np.radians(half_y_deg) * t
    th = np.pi / 2 + np.radians(half_z_deg) * t
    P, T = np.meshgrid(ph, th, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], axis=-1).reshape(-1, 3)
    if frame is not None:
        d = d @ np.asarray(frame).T
    out = np.zeros((d.shape[0], 6))
    out[:, 3:] = d
    return out


def velocity_particles(records: np.ndarray, n: int, seed: int = 5, v_rms: float = 1e-3) -> tuple:
    """Synthetic particles for the velocity-field deposit: positions (n x 3,
    float32, octree units) drawn cell by cell (a uniformly chosen leaf cell,
    then uniformly inside it, so refined regions get more particles per unit
    volume), velocities (n x 3, float32, in units of c) along minus the
    potential gradient of their cell, scaled to an rms of v_rms, plus 20 %
    isotropic noise: the linear-theory flow toward the potential wells."""
    rng = np.random.default_rng(seed)
    lev = key_level(records["hi"], records["lo"]).astype(np.int64)
    # leaves: cells with no next key inside them (pre-order sort: a child follows its parent)
    nxt_level = np.append(lev[1:], 0)
    leaf = np.flatnonzero(nxt_level <= lev)
    pick = leaf[rng.integers(0, leaf.shape[0], n)]
    centers = np.zeros((n, 3))
    for L in np.unique(lev[pick]):
        m = lev[pick] == L
        c = key_coords(records["hi"][pick[m]], records["lo"][pick[m]], int(L))
        centers[m] = cell_center(int(L), c)
    size = 4.0 / 2.0 ** lev[pick]
    pos = centers + rng.uniform(-0.5, 0.5, (n, 3)) * size[:, None]
    g = np.stack([records["dphidx"][pick], records["dphidy"][pick], records["dphidz"][pick]], axis=1).astype(np.float64)
    gn = np.sqrt((g ** 2).sum(1).mean()) or 1.0
    vel = -g / gn * v_rms + rng.normal(0.0, 0.2 * v_rms / np.sqrt(3.0), (n, 3))
    return pos.astype(np.float32), vel.astype(np.float32)
