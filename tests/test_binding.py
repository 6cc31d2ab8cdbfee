"""The binding a BEEP maintainer adds (beep_gb300/binding/beep_binding.*):
ModelPack / TablePack pack BEEP's own Data, Model, ObservationModel and the
tables of State::set_param into beep_model_desc / beep_param_tables.  The
golden fixtures are written through it by the reference harness; here a
fixture is regenerated from the reference and compared with the committed
one array for array, so the packing every GPU parity test consumes is the
binding's.  Needs the reference tree (skipped where it is absent)."""
import os
import sys

import numpy as np
import pytest

from beep_gb300 import bundle, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


@pytest.mark.skipif(not os.path.exists(HARNESS), reason="the reference harness is built only where the reference tree is")
def test_fixture_through_the_binding_equals_the_committed_one(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    w = synth.seir_hd_features()
    make_golden.make_fixture("features_sim", w, npart=8, ntraj=2, seed=0xFEA7, outdir=str(tmp_path))
    new = bundle.read_bundle(os.path.join(str(tmp_path), "features_sim.bnd"))
    old = bundle.read_bundle(os.path.join(ROOT, "tests", "golden", "features_sim.bnd"))
    assert set(old) <= set(new)
    for k in old:
        if k == "obs_shape":      # the reference leaves Observation::shape unset for normal models
            continue
        assert np.array_equal(old[k], new[k]), k
