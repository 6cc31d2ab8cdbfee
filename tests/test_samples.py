"""Sample files of a sampled particle-filter lineage, written by
beep_gb300.samples, against the files the reference itself wrote for the same
lineage (tests/golden/tiny_pf_sample*, from Mpi::gather_samples / State::save)."""
import os

import numpy as np

from beep_gb300 import samples
from golden_util import GOLDEN, load


def test_sample_files_match_reference(tmp_path):
    b, m, tabs, seed = load("tiny_pf")
    ref_par = open(os.path.join(GOLDEN, "tiny_pf_sample0_parameter.csv")).read()
    names = [line.split(",")[0] for line in ref_par.splitlines()[2:]]
    times = samples.division_times(m.period, m.ndivision, start=0.0)
    samples.write_sample(str(tmp_path), 0, float(b["g0.pf.lineage_EF"][0]), names, b["g0.theta"],
                         b["g0.pf.lineage_transnum"], times)
    samples.write_sample_information(str(tmp_path), 1, "tiny70.toml", "0", "70", m.division_per_time, m.ndivision)
    for f in ("sample0_parameter.csv", "sample0_transition.csv", "sample_information.txt"):
        assert open(os.path.join(tmp_path, f)).read() == open(os.path.join(GOLDEN, "tiny_pf_" + f)).read(), f


def test_number_format_follows_cpp_streams():
    assert samples.fmt(4.0) == "4"
    assert samples.fmt(-19570.78023191) == "-19570.8"
    assert samples.fmt(1234567.0) == "1.23457e+06"
    assert samples.fmt(0.125) == "0.125"
    assert samples.fmt(1e-5) == "1e-05"
    assert np.allclose(samples.division_times(70, 280)[:2], [0.125, 0.375])
