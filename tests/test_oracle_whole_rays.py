"""CPU tests: the C oracle on whole rays of the two parity workloads (the
benchmark octree's AMR construction at a small size, to z = 2, and the
uniform 64^3 cone along phi = theta = 20 degrees, to z = 0.5) against the
reference's own Integrator::integrate on the same octrees
(tests/golden/whole_rays.npz): step counts and every field of the final
photon records bit-identical.  The octrees are regenerated from their seeds
and checked against the recorded hash first."""
import importlib
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

sys.path.insert(0, GOLDEN)
MG = importlib.import_module("make_golden")


@pytest.fixture(scope="module")
def whole():
    return load_golden("whole_rays")


@pytest.mark.parametrize("name,order", [("amr_z2", 1), ("amr_z2", 2), ("cone20_z05", 1)])
def test_oracle_whole_rays_bit_exact(whole, synth, oracle_mod, name, order):
    spec, _, zstop, nsteps, _ = MG.whole_rays_specs()[name]
    rec = synth.make_octree(spec)
    assert MG.records_sha(rec) == str(whole[name + "_sha"]), "the seeded octree differs from the fixture's"
    table = synth.Cosmology().conformal_table(n=4000, amin=0.05)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    O = oracle_mod.Oracle(rec, {"t": table[0], "a": table[1], "dadt": table[2]}, length)
    steps, final, _ = O.propagate(whole[name + "_launch"], order=order, nsteps=nsteps, stop="redshift", stop_ref=zstop)
    np.testing.assert_array_equal(steps, whole["%s_steps_o%d" % (name, order)])
    np.testing.assert_array_equal(final.view(np.uint64), whole["%s_final_o%d" % (name, order)].view(np.uint64))
