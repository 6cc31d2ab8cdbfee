// Binding of BEEP's State::simulate to the GB300 library: packing of BEEP's
// own objects into beep_model_desc / beep_param_tables (see beep_binding.hh).
// Compiled inside BEEP's source tree, against BEEP's headers.
#include "beep_binding.hh"

#include <algorithm>
#include <map>

#include "data.hh"
#include "details.hh"
#include "model.hh"
#include "obsmodel.hh"
#include "state.hh"

namespace beep_binding {

ModelPack::ModelPack(const Details &details, const Data &data, const Model &model)
{
	const unsigned A = data.narea, DP = data.ndemocatpos, C = model.comp.size(), T = model.trans.size();
	const unsigned DPS = data.ndemocatpos_per_strain;
	for (unsigned tr = 0; tr < T; tr++) {
		trans_from.push_back((int32_t)model.trans[tr].from);
		trans_to.push_back((int32_t)model.trans[tr].to);
	}
	for (unsigned dp = 0; dp < DPS; dp++) democatpos_age.push_back((int32_t)data.democatpos[dp][0]);
	// area mixing as the reference stores it: diagonal, off-diagonal rows genQ.M, genQ.factor
	M_rowptr.assign(A + 1, 0);
	for (unsigned c = 0; c < A; c++) {
		M_diag.push_back(data.genQ.M.diag[c]);
		M_factor.push_back(data.genQ.factor[c]);
		for (unsigned j = 0; j < data.genQ.M.to[c].size(); j++) {
			M_to.push_back((int32_t)data.genQ.M.to[c][j]);
			M_val.push_back(data.genQ.M.val[c][j]);
		}
		M_rowptr[c + 1] = (int32_t)M_to.size();
	}
	pop_init.resize((size_t)A * C * DP);
	for (unsigned c = 0; c < A; c++)
		for (unsigned co = 0; co < C; co++)
			for (unsigned dp = 0; dp < DP; dp++) pop_init[((size_t)c * C + co) * DP + dp] = data.area[c].pop_init[co][dp];
	// observations; each one's cells in the order get_obs_value_section visits them
	// (src/obsmodel.cc:74-109): area, transitions before populations, transition or
	// compartment, demographic position
	std::map<unsigned, int32_t> spline_row;
	const unsigned nobs = data.nobs;
	obs_cell_ptr.assign(nobs + 1, 0);
	for (unsigned i = 0; i < nobs; i++) {
		const auto &ob = data.obs[i];
		obs_sett_i.push_back((int32_t)ob.sett_i);
		obs_sett_f.push_back((int32_t)ob.sett_f);
		obs_value_kind.push_back(ob.value == UNKNOWN ? BEEP_OBSVAL_UNKNOWN : (ob.value == THRESH ? BEEP_OBSVAL_THRESH : BEEP_OBSVAL_VALUE));
		obs_value.push_back(ob.value);
		obs_sd.push_back(ob.sd);
		obs_shape.push_back(ob.shape);
		obs_threshold.push_back(data.datatable[ob.datatable].threshold);
		obs_factor.push_back(ob.factor);
		obs_model.push_back((int32_t)ob.obsmodel);
		if (ob.factor_spline == UNSET) obs_factor_spline.push_back(-1);
		else {
			if (!spline_row.count(ob.factor_spline)) {
				spline_row[ob.factor_spline] = (int32_t)obs_spline_refs.size();
				obs_spline_refs.push_back(ob.factor_spline);
			}
			obs_factor_spline.push_back(spline_row[ob.factor_spline]);
		}
		struct Cell {
			unsigned c, kind, x, dp;
			int32_t cell;
		};
		std::vector<Cell> ks;
		const auto &dtab = data.datatable[ob.datatable];
		for (auto c : ob.area)
			for (auto dp : ob.dp_sel) {
				for (auto tr : dtab.translist) ks.push_back({c, 0, tr, dp, (int32_t)((c * T + tr) * DP + dp)});
				for (auto co : dtab.complist) ks.push_back({c, 1, co, dp, (int32_t)(-1 - (int32_t)((c * C + co) * DP + dp))});
			}
		std::stable_sort(ks.begin(), ks.end(), [](const Cell &a, const Cell &b) {
			if (a.c != b.c) return a.c < b.c;
			if (a.kind != b.kind) return a.kind < b.kind;
			if (a.x != b.x) return a.x < b.x;
			return a.dp < b.dp;
		});
		for (auto &k : ks) obs_cells.push_back(k.cell);
		obs_cell_ptr[i + 1] = (int32_t)obs_cells.size();
	}
	desc.narea = (int32_t)A; desc.nage = (int32_t)data.nage; desc.ndemocatpos = (int32_t)DP;
	desc.nstrain = (int32_t)data.nstrain; desc.ncomp = (int32_t)C; desc.ntrans = (int32_t)T;
	desc.ndivision = (int32_t)details.ndivision; desc.period = (int32_t)details.period;
	desc.division_per_time = (int32_t)details.division_per_time;
	desc.dt = double(details.period) / details.ndivision;
	desc.popsize = (double)data.popsize;
	desc.trans_from = trans_from.data(); desc.trans_to = trans_to.data();
	desc.infection_trans = (int32_t)model.infection_trans;
	desc.democatpos_age = democatpos_age.data();
	desc.M_diag = M_diag.data(); desc.M_rowptr = M_rowptr.data(); desc.M_to = M_to.data(); desc.M_val = M_val.data();
	desc.M_factor = M_factor.data(); desc.pop_init = pop_init.data();
	desc.nobs = (int32_t)nobs;
	desc.obs_sett_i = obs_sett_i.data(); desc.obs_sett_f = obs_sett_f.data();
	desc.obs_value_kind = obs_value_kind.data(); desc.obs_value = obs_value.data(); desc.obs_model = obs_model.data();
	desc.obs_sd = obs_sd.data(); desc.obs_shape = obs_shape.data(); desc.obs_threshold = obs_threshold.data();
	desc.obs_factor = obs_factor.data(); desc.obs_factor_spline = obs_factor_spline.data();
	desc.obs_cell_ptr = obs_cell_ptr.data(); desc.obs_cells = obs_cells.data();

	// demographic changes: areas, dp groups and per-step fractions as loaded by
	// Data::load_democat_change (src/data.cc:958-1040)
	dcc_area_ptr.push_back(0);
	dcc_dp_ptr.push_back(0);
	for (const auto &dcc : data.democat_change) {
		const unsigned nv = dcc.frac.empty() ? 0 : dcc.frac[0].size();
		dcc_nval.push_back((int32_t)nv);
		for (auto c : dcc.area) dcc_area.push_back((int32_t)c);
		dcc_area_ptr.push_back((int32_t)dcc_area.size());
		for (const auto &grp : dcc.dp_group)
			for (auto dp : grp) dcc_dp.push_back((int32_t)dp);
		dcc_dp_ptr.push_back((int32_t)dcc_dp.size());
		for (unsigned s = 0; s < details.ndivision; s++)
			for (unsigned f = 0; f < nv; f++) dcc_frac.push_back(dcc.frac[s][f]);
	}
	desc.ndemocat_change = (int32_t)data.democat_change.size();
	if (desc.ndemocat_change > 0) {
		desc.dcc_nval = dcc_nval.data(); desc.dcc_area_ptr = dcc_area_ptr.data(); desc.dcc_area = dcc_area.data();
		desc.dcc_dp_ptr = dcc_dp_ptr.data(); desc.dcc_dp = dcc_dp.data(); desc.dcc_frac = dcc_frac.data();
	}
}

TablePack::TablePack(const ModelPack &mp, const Details &details, const Data &data, const Model &model,
                     const State &state, const std::vector<double> &paramval)
{
	const unsigned A = data.narea, G = data.nage, DP = data.ndemocatpos, NS = data.nstrain;
	const unsigned C = model.comp.size(), T = model.trans.size(), S = details.ndivision;
	for (unsigned tr = 0; tr < T; tr++) {
		if (state.transrate[tr].size() == DP) transrate.insert(transrate.end(), state.transrate[tr].begin(), state.transrate[tr].end());
		else transrate.insert(transrate.end(), DP, 0.0);   // the infection transition has no rate
	}
	susceptibility = state.susceptibility;
	for (unsigned co = 0; co < C; co++) infectivity.push_back(paramval[model.comp[co].infectivity_param]);
	// beta rows, one per distinct row (the reference copies one row per R-spline to its
	// areas, src/model.cc:1339-1345), and the row of each (strain, area)
	std::vector<const std::vector<double> *> rows;
	beta_row_of.resize((size_t)NS * A);
	for (unsigned st = 0; st < NS; st++)
		for (unsigned c = 0; c < A; c++) {
			const auto &r = state.beta[st][c];
			unsigned k = 0;
			while (k < rows.size() && *rows[k] != r) k++;
			if (k == rows.size()) rows.push_back(&r);
			beta_row_of[st * A + c] = (int32_t)k;
		}
	for (auto *r : rows) beta_rows.insert(beta_rows.end(), r->begin(), r->end());
	for (unsigned t = 0; t < details.period; t++) areafactor.insert(areafactor.end(), state.areafactor[t].begin(), state.areafactor[t].end());
	for (unsigned s = 0; s < S; s++)
		for (unsigned a = 0; a < G; a++) Ntime.insert(Ntime.end(), state.Ntime[s][a].begin(), state.Ntime[s][a].end());
	geo_spline = state.disc_spline[model.geo_spline_ref];
	for (auto &info : model.efoispline_info) {
		efoi_spline.insert(efoi_spline.end(), state.disc_spline[info.spline_ref].begin(), state.disc_spline[info.spline_ref].end());
		efoi_agedist.insert(efoi_agedist.end(), info.efoi_agedist.begin(), info.efoi_agedist.end());
	}
	for (unsigned st = 0; st < NS; st++)
		for (unsigned c = 0; c < A; c++) efoi_ref.push_back((int32_t)model.efoi_spl_ref[st][c]);
	for (auto spl : mp.obs_spline_refs) obs_spline.insert(obs_spline.end(), state.disc_spline[spl].begin(), state.disc_spline[spl].end());
	if (details.mode == PREDICTION) {                 // model modifications (ModelMod)
		for (unsigned s = 0; s < S; s++)
			for (unsigned c = 0; c < A; c++) {
				for (unsigned st = 0; st < NS; st++) efoi_mult.push_back(model.modelmod.efoi_mult[s][c][st]);
				for (unsigned tr = 0; tr < T; tr++)
					for (unsigned dp = 0; dp < DP; dp++) transmean_mult.push_back(model.modelmod.transmean_mult[s][c][tr][dp]);
			}
	}
	tables.transrate = transrate.data();
	tables.susceptibility = susceptibility.data();
	tables.infectivity = infectivity.data();
	tables.nbeta_row = (int32_t)rows.size();
	tables.beta_rows = beta_rows.data();
	tables.beta_row_of = beta_row_of.data();
	tables.areafactor = areafactor.data();
	tables.Ntime = Ntime.data();
	tables.geo_spline = geo_spline.data();
	tables.nefoi = (int32_t)model.efoispline_info.size();
	tables.efoi_spline = efoi_spline.data();
	tables.efoi_agedist = efoi_agedist.data();
	tables.efoi_ref = efoi_ref.data();
	tables.nobs_spline = (int32_t)mp.obs_spline_refs.size();
	tables.obs_spline = obs_spline.data();
	tables.efoi_mult = efoi_mult.empty() ? nullptr : efoi_mult.data();
	tables.transmean_mult = transmean_mult.empty() ? nullptr : transmean_mult.data();
}

PriorPack::PriorPack(const Details &details, const Model &model)
{
	const unsigned np = model.param.size();
	auto par_or_none = [&](unsigned p) { return p < np ? (int32_t)p : -1; };
	gt_ptr.push_back(0);
	lt_ptr.push_back(0);
	for (unsigned th = 0; th < np; th++) {
		const auto &par = model.param[th];
		type.push_back((int32_t)par.priortype);
		val1.push_back(par.val1);
		val2.push_back(par.val2);
		val1_param.push_back(par_or_none(par.val1_param));
		val2_param.push_back(par_or_none(par.val2_param));
		for (auto t2 : par.greaterthan) gt_param.push_back((int32_t)t2);
		for (auto t2 : par.lessthan) lt_param.push_back((int32_t)t2);
		gt_ptr.push_back((int32_t)gt_param.size());
		lt_ptr.push_back((int32_t)lt_param.size());
	}
	dir_ptr.push_back(0);
	for (const auto &dir : model.dirichlet) {
		for (const auto &dp : dir.param) {
			dir_param.push_back((int32_t)dp.th);
			dir_frac.push_back(dp.frac);
		}
		dir_ptr.push_back((int32_t)dir_param.size());
	}
	// the consecutive spline points Model::spline_prior smooths (none when simulating)
	if (details.siminf != SIMULATE)
		for (const auto &spl : model.spline) {
			if (spl.smoothtype == NOSMOOTH) continue;
			for (unsigned i = 0; i + 1 < spl.p.size(); i++) {
				const auto &a = spl.p[i], &b = spl.p[i + 1];
				if (a.param == b.param || a.t == b.t) continue;
				if (model.param[a.param].priortype == FIXED_PRIOR && model.param[b.param].priortype == FIXED_PRIOR) continue;
				smooth_kind.push_back(spl.smoothtype == LOGSMOOTH ? 1 : 2);
				smooth_par1.push_back((int32_t)a.param);
				smooth_par2.push_back((int32_t)b.param);
				smooth_mult1.push_back(a.multfac);
				smooth_mult2.push_back(b.multfac);
				smooth_value.push_back(a.smooth_value);
			}
		}
	spec.nparam = (int32_t)np;
	spec.type = type.data(); spec.val1 = val1.data(); spec.val2 = val2.data();
	spec.val1_param = val1_param.data(); spec.val2_param = val2_param.data();
	spec.gt_ptr = gt_ptr.data(); spec.gt_param = gt_param.data(); spec.lt_ptr = lt_ptr.data(); spec.lt_param = lt_param.data();
	spec.ndirichlet = (int32_t)model.dirichlet.size();
	spec.dir_ptr = dir_ptr.data(); spec.dir_param = dir_param.data(); spec.dir_frac = dir_frac.data();
	spec.nsmooth = (int32_t)smooth_kind.size();
	spec.smooth_kind = smooth_kind.data(); spec.smooth_par1 = smooth_par1.data(); spec.smooth_par2 = smooth_par2.data();
	spec.smooth_mult1 = smooth_mult1.data(); spec.smooth_mult2 = smooth_mult2.data(); spec.smooth_value = smooth_value.data();
	spec.ml_mode = details.mode == ML_INF ? 1 : 0;
}

}  // namespace beep_binding
