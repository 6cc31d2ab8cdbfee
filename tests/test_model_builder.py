"""The host restatement of State::set_param and the model set-up
(beep_gb300/model_builder.py: Model::create_transrate, create_disc_spline,
create_susceptibility, create_areafactor, create_Ntime, calculate_beta_from_R,
src/model.cc:1010-1362; Data::geo_normalise and the age-matrix normalisation,
src/data_matrix.cc:55-202) against the arrays the compiled reference itself
produced for the golden fixtures' workloads."""
import numpy as np
import pytest

from beep_gb300 import model_builder as mb, synth
from golden_util import load

WORKLOADS = {
    "tiny_sim": lambda: synth.seir_hd_small(seed=20260100, narea=4, nage=3, days=40, name="tiny"),
    "oneage_sim": lambda: synth.seir_hd_small(seed=20260101, narea=5, nage=1, days=30, name="oneage"),
    "c0_sim": lambda: synth.seir_hd_small(seed=20260000, narea=10, nage=3, days=100, name="c0"),
    # area covariates, stepped age-mixing factors, external force of infection, 7-knot R(t)
    "features_sim": synth.seir_hd_features,
    # two strains: susceptibility and R factor per strain, one NGM per strain
    "strain_sim": synth.seir_hd_strains,
    "strain70_model": lambda: synth.seir_hd_strains(narea=70, nage=2, days=20, name="strains70"),
    # demographic changes of the age distribution (all areas, and a geo filter)
    "democat_sim": synth.seir_hd_democat,
}
DCC_KEYS = ("dcc_nval", "dcc_area_ptr", "dcc_area", "dcc_dp_ptr", "dcc_dp", "dcc_frac")
MODEL_KEYS = ("dims", "trans_from", "trans_to", "democatpos_age", "M_diag", "M_rowptr", "M_to", "M_val", "M_factor",
              "pop_init", "obs_sett_i", "obs_sett_f", "obs_cell_ptr", "obs_cells", "obs_factor")
TABLE_KEYS = ("transrate", "susceptibility", "infectivity", "beta_rows", "beta_row_of", "areafactor", "Ntime",
              "geo_spline", "efoi_spline", "efoi_agedist", "efoi_ref")


def _close(x, y):
    x, y = np.asarray(x, np.float64).ravel(), np.asarray(y, np.float64).ravel()
    assert x.shape == y.shape
    np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_model_and_tables_match_reference(name):
    b, _, _, _ = load(name)
    w = WORKLOADS[name]()
    arr = mb.model_arrays(w)
    for k in MODEL_KEYS:
        _close(arr[k], b[k])
    for k in DCC_KEYS:
        assert (k in arr) == (k in b), k
        if k in b:
            _close(arr[k], b[k])
    t = mb.param_tables(w)
    for k in TABLE_KEYS:
        _close(t[k], b["g0." + k])


def test_observations_match_reference_for_every_observation_model():
    """The observation list of the workload observed through every model the
    reference parses (normal X%, Poisson with censoring below a threshold,
    fixed-SD normal, loaded SDs with a threshold, missing entries): values,
    kinds, models, standard deviations (Data::set_obs_sd, src/data.cc:1589-1623)
    and thresholds equal the reference's."""
    b, _, _, _ = load("obsmodel_sim")
    w = synth.seir_hd_obs_models()
    # the observed values as the data files carried them: censored entries are below
    # the threshold, missing ones any value
    val, kind, sd = (np.asarray(b[k]) for k in ("obs_value", "obs_value_kind", "obs_sd"))
    ov, k = {}, 0
    for tab in synth.data_tables(w):
        n = len(tab["times"])
        ov[tab["file"]] = {}
        for col in tab["columns"]:
            ov[tab["file"]][col] = (np.where(kind[k:k + n] == 0, val[k:k + n], 0.0),
                                    sd[k:k + n] if tab.get("sd_col", True) else None)
            k += n
    arr = mb.model_arrays(w, ov)
    for key in MODEL_KEYS + ("obs_value_kind", "obs_value", "obs_model", "obs_sd", "obs_threshold"):
        _close(arr[key], b[key])
