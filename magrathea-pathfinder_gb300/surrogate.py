"""Learned field surrogate (host side): a per-cone Fourier-feature MLP trained
on the octree's TSC field and used in place of the octree gather inside the
RK4 stages, with the octree as check and fallback.  Compute in
libmpf_gb300.so (mpf_surrogate_* in include/mpf_gb300.h).

    s = Surrogate(cone_tan=(ty, tz), r_max=..., a_min=...)
    s.train(octree, samples=50_000_000)
    steps, final, flags, drift, stats = s.propagate(octree, cosmology, launch, length, stop="redshift",
                                                     stop_value=2.0)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import MPF_PHOTON_FIELDS, MPF_SURROGATE_NORM, MPF_SURROGATE_PARAMS


class Surrogate:
    def __init__(self, cone_tan, r_max: float, a_min: float, a_max: float = 1.0, r_min: float = 0.0,
                 freq_sigma=(8.0, 2.0, 2.0, 1.0), seed: int = 42):
        L = capi.load()
        d = capi.SurrogateDomain()
        d.tan_half[0], d.tan_half[1] = float(cone_tan[0]), float(cone_tan[1])
        d.r_min, d.r_max, d.a_min, d.a_max = float(r_min), float(r_max), float(a_min), float(a_max)
        for q in range(4):
            d.freq_sigma[q] = float(freq_sigma[q])
        d.seed = int(seed)
        h = C.c_void_p()
        capi.check(L.mpf_surrogate_create(C.byref(d), C.byref(h)))
        self._h = h
        self._lib = L

    # -- parameters -------------------------------------------------------
    def get_params(self):
        p = np.zeros(MPF_SURROGATE_PARAMS, dtype=np.float32)
        n = np.zeros(MPF_SURROGATE_NORM, dtype=np.float32)
        capi.check(self._lib.mpf_surrogate_get_params(self._h, capi.ptr(p), capi.ptr(n)))
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        if p is not None and p.shape != (MPF_SURROGATE_PARAMS,):
            raise ValueError("expected %d parameters" % MPF_SURROGATE_PARAMS)
        if n is not None and n.shape != (MPF_SURROGATE_NORM,):
            raise ValueError("expected %d normalisation values" % MPF_SURROGATE_NORM)
        capi.check(self._lib.mpf_surrogate_set_params(self._h, capi.ptr(p), capi.ptr(n)))

    # -- training ---------------------------------------------------------
    def sample(self, octree, n: int, first: int = 0):
        x = np.zeros((n, 4), dtype=np.float32)
        t = np.zeros((n, 5), dtype=np.float32)
        capi.check(self._lib.mpf_surrogate_sample(self._h, octree._h, int(first), n, capi.ptr(x), capi.ptr(t)))
        return x, t

    def loss_grad(self, inputs, targets):
        x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 5)
        g = np.zeros(MPF_SURROGATE_PARAMS, dtype=np.float32)
        loss = C.c_double()
        capi.check(self._lib.mpf_surrogate_loss_grad(self._h, x.shape[0], capi.ptr(x), capi.ptr(t), C.byref(loss),
                                                     capi.ptr(g)))
        return loss.value, g

    def train(self, octree, samples: int = 50_000_000, batch: int = 16384, lr: float = 2e-3,
              stat_samples: int = 262144) -> dict:
        p = capi.SurrogateTrainParams()
        p.samples, p.batch, p.lr, p.stat_samples = int(samples), int(batch), float(lr), int(stat_samples)
        st = capi.SurrogateTrainStats()
        capi.check(self._lib.mpf_surrogate_train(self._h, octree._h, C.byref(p), C.byref(st)))
        return dict(loss_first=st.loss_first, loss_last=st.loss_last, steps=st.steps, seconds=st.seconds,
                    samples_per_second=st.samples_per_second, kernel_launches_per_step=st.kernel_launches_per_step)

    # -- inference --------------------------------------------------------
    def eval(self, inputs) -> np.ndarray:
        """phi dphidx dphidy dphidz dphidt at (x, y, z, a) rows, through the tensor-core path."""
        x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, 4)
        out = np.zeros((x.shape[0], 5), dtype=np.float32)
        capi.check(self._lib.mpf_surrogate_eval(self._h, x.shape[0], capi.ptr(x), capi.ptr(out)))
        return out

    def propagate(self, octree, cosmology, launch, length: float, nsteps: int = 10, order: int = 2,
                  stop: str = "redshift", stop_value: float = 0.0, max_steps: int = 0, tolerance: float = 1e-3,
                  check_every: int = 64, fallback: bool = True, want_final: bool = True):
        """Returns (steps[n], final[n, 28] or None, flags[n], drift[n], stats dict)."""
        launch = np.ascontiguousarray(launch, dtype=np.float64).reshape(-1, 6)
        n = launch.shape[0]
        p, keep = capi.make_params(length, nsteps, order, stop, stop_value, None, False, False, max_steps)
        sp = capi.SurrogatePropParams()
        sp.tolerance, sp.check_every, sp.fallback = float(tolerance), int(check_every), int(bool(fallback))
        steps = np.zeros(n, dtype=np.int64)
        final = np.zeros((n, MPF_PHOTON_FIELDS)) if want_final else None
        flags = np.zeros(n, dtype=np.uint8)
        drift = np.zeros(n, dtype=np.float32)
        st = capi.SurrogatePropStats()
        rc = self._lib.mpf_surrogate_propagate(self._h, octree._h, cosmology._h, C.byref(p), C.byref(sp), n,
                                               capi.ptr(launch), capi.ptr(steps), capi.ptr(final), capi.ptr(flags),
                                               capi.ptr(drift), C.byref(st))
        capi.check(rc)
        del keep
        stats = dict(photon_steps=st.photon_steps, flagged_photons=st.flagged_photons,
                     fallback_photons=st.fallback_photons, fallback_steps=st.fallback_steps,
                     surrogate_seconds=st.surrogate_seconds, fallback_seconds=st.fallback_seconds)
        return steps, final, flags, drift, stats

    def close(self):
        if self._h:
            self._lib.mpf_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
