// Binding of BEEP's State::simulate to the GB300 library (include/beep_gpu.h).
//
// This is the code a BEEP maintainer adds to BEEP's own source tree: it
// includes BEEP's headers and reads the objects BEEP has already built
// (Details, Data, Model, ObservationModel after src/main.cc:125-160, and a
// State after State::set_param), so that the hot path -- State::simulate plus
// ObservationModel::calculate(_section) -- runs on the GPU instead:
//
//   beep_binding::ModelPack mp(details, data, model);      // once per run
//   beep_model *gm;  beep_model_create(&mp.desc, &gm);
//   state.set_param(paramval);                              // BEEP's own tables
//   beep_binding::TablePack tp(mp, details, data, model, state, paramval);
//   beep_binding::simulate(gm, tp, N, seed, ti, tf, ...);   // State::simulate(ti, tf) of N particles
//
// Every array is packed in the layout and order the reference itself uses:
// the area mixing as BEEP's genQ.M rows, observation cells in the order
// ObservationModel::get_obs_value_section visits them (src/obsmodel.cc:74-109),
// transition rates, splines, area factors and age-mixing tables as set_param
// left them (src/model.cc:1010-1362), and, in prediction mode, the model
// modifications' multipliers (ModelMod, src/model.cc:1446-1585).  The golden
// fixtures of the test suite are written through these two classes, so every
// GPU parity test exercises this binding's packing.
#pragma once

#include <cstdint>
#include <vector>

#include "beep_gpu.h"

class Details;
class Data;
class Model;
class ObservationModel;
class State;

namespace beep_binding {

// The parameter-independent model (beep_model_desc): arrays owned here, desc points into them.
struct ModelPack {
	std::vector<int32_t> trans_from, trans_to, democatpos_age, M_rowptr, M_to;
	std::vector<double> M_diag, M_val, M_factor, pop_init;
	std::vector<int32_t> obs_sett_i, obs_sett_f, obs_value_kind, obs_model, obs_factor_spline, obs_cell_ptr, obs_cells;
	std::vector<double> obs_value, obs_sd, obs_shape, obs_threshold, obs_factor;
	std::vector<unsigned> obs_spline_refs;   // BEEP spline index of each observation-factor spline row
	std::vector<int32_t> dcc_nval, dcc_area_ptr, dcc_area, dcc_dp_ptr, dcc_dp;   // Data::democat_change
	std::vector<double> dcc_frac;
	beep_model_desc desc{};

	ModelPack(const Details &details, const Data &data, const Model &model);
	ModelPack(const ModelPack &) = delete;
	ModelPack &operator=(const ModelPack &) = delete;
};

// The tables State::set_param produced for one parameter set (beep_param_tables).
struct TablePack {
	std::vector<double> transrate, susceptibility, infectivity, beta_rows, areafactor, Ntime, geo_spline, efoi_spline,
	    efoi_agedist, obs_spline, efoi_mult, transmean_mult;
	std::vector<int32_t> beta_row_of, efoi_ref;
	beep_param_tables tables{};

	TablePack(const ModelPack &mp, const Details &details, const Data &data, const Model &model, const State &state,
	          const std::vector<double> &paramval);
	TablePack(const TablePack &) = delete;
	TablePack &operator=(const TablePack &) = delete;
};

// The priors and bounds of BEEP's parameters (beep_prior_spec): Param's prior
// type, hyperparameters and order constraints, the Dirichlet groups, and the
// spline smoothing terms Model::spline_prior evaluates.
struct PriorPack {
	std::vector<int32_t> type, val1_param, val2_param, gt_ptr, gt_param, lt_ptr, lt_param, dir_ptr, dir_param,
	    smooth_kind, smooth_par1, smooth_par2;
	std::vector<double> val1, val2, dir_frac, smooth_mult1, smooth_mult2, smooth_value;
	beep_prior_spec spec{};

	PriorPack(const Details &details, const Model &model);
	PriorPack(const PriorPack &) = delete;
	PriorPack &operator=(const PriorPack &) = delete;
};

// State::simulate(ti, tf) + ObservationModel::calculate(_section) for nparticle
// particles of one parameter set (particle p on variate stream p): pop_in
// [nparticle][narea][ncomp][ndemocatpos] when ti > 0; L_out [nparticle],
// pop_out (same layout as pop_in) and transnum_out
// [nparticle][tf-ti][narea][ntrans][ndemocatpos] may be null.  form is a beep_form.
// (Models with demographic changes pass FP64 populations: the overload below.)
inline beep_status simulate(beep_model *gm, const TablePack &t, int32_t nparticle, uint64_t seed, int32_t ti,
                            int32_t tf, const int32_t *pop_in, double *L_out, int32_t *pop_out, int32_t *transnum_out,
                            int32_t form)
{
	beep_sim_batch b{};
	b.nparticle = nparticle;
	b.ngroup = 1;
	b.groups = &t.tables;
	b.seed = seed;
	b.ti = ti;
	b.tf = tf;
	b.pop_in = pop_in;
	b.L_out = L_out;
	b.pop_out = pop_out;
	b.transnum_out = transnum_out;
	b.form = form;
	return beep_simulate(gm, &b);
}

// The same for a model with demographic changes: populations are FP64, as in State::pop.
inline beep_status simulate(beep_model *gm, const TablePack &t, int32_t nparticle, uint64_t seed, int32_t ti,
                            int32_t tf, const double *pop_in, double *L_out, double *pop_out, int32_t *transnum_out)
{
	beep_sim_batch b{};
	b.nparticle = nparticle;
	b.ngroup = 1;
	b.groups = &t.tables;
	b.seed = seed;
	b.ti = ti;
	b.tf = tf;
	b.pop_in_f64 = pop_in;
	b.L_out = L_out;
	b.pop_out_f64 = pop_out;
	b.transnum_out = transnum_out;
	b.form = BEEP_FORM_PLAIN_FP64;
	return beep_simulate(gm, &b);
}

}  // namespace beep_binding
