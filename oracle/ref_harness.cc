// ref_harness.cc -- drives the compiled reference (BEEP's own C++ sources,
// built in place from the reference tree by oracle/Makefile.ref) to produce
// golden vectors.  TEST INFRASTRUCTURE ONLY.
//
// It builds Inputs -> Details -> Mpi -> Data -> Model -> ObservationModel as
// src/main.cc:125-160 does, then for each particle calls State::simulate(θ)
// (src/state.cc:582-592), and, for particle-filter sections, the sectioned
// State::simulate(ti,tf) + ObservationModel::calculate_section
// (src/state.cc:596-638, src/obsmodel.cc:39-58).  Every poisson_sample call
// (src/utils.cc:148-153) is interposed at link time (-Wl,--wrap) and answered
// from the project's keyed Philox stream, so the reference consumes exactly
// the variates the oracle restatement and the CUDA kernels consume.
//
// It writes one bundle file: the parameter-independent model, the tables
// set_param produced, and the reference's outputs (log-likelihoods,
// transition counts and populations).
//
// With mbp=N it also drives the reference's Mbp (src/mbp.cc:252-361): N
// chains, each simulated at one parameter row and proposed at the next, with
// binomial_sample (src/utils.cc:174-180) interposed like poisson_sample.
//
// With abcw=N abck=K it evaluates the reference's ABC-SMC importance weights
// (ABCSMC::calculate_particle_weight, normalise_particle_weights and the
// weighted MVN, src/abcsmc.cc:260-283, src/mvn.cc:39-196): parameter rows
// 0..K-1 form the previous generation (weights 0.5 + 0.1 (j mod 7)), rows
// K..K+N-1 are the new samples; BEEP's own inputs need nsample and ngeneration.
//
// With pred=DIR predn=K (BEEP's mode=prediction with modifications) it loads the
// posterior samples DIR/sample0..K-1 and simulates each from the modifications'
// start to the end, as the reference's prediction mode does.
//
// usage: ref_harness out=FILE [npart=N] [ntraj=N] [seed=S] [pf=0|1] [theta=FILE] [mbp=N] [sampledir=DIR]
//                    [abcw=N abck=K] [pred=DIR predn=K] -- <BEEP key=value...>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#include <algorithm>

#include "inputs.hh"
#include "details.hh"
#include "output.hh"
// The particle-filter driver below calls the reference's own private
// PMCMC::bootstrap; the access specifiers are lifted for this translation unit.
#define private public
#include "pmcmc.hh"
#include "mbp.hh"
#include "abcsmc.hh"
#undef private
#include "mpi.hh"
#include "data.hh"
#include "model.hh"
#include "obsmodel.hh"
#include "state.hh"
#include "utils.hh"
#include "timers.hh"

#include "beep_binding.hh"

extern "C" {
#include "beep_rng_ref.h"
}

// ---- replay hook ---------------------------------------------------------

namespace {
struct Replay {
	bool active = false;
	const State *st = nullptr;
	// Mbp::mbp replay: st is the proposed state, ini the initial one
	bool mbp = false;
	const State *ini = nullptr;
	const std::vector<std::vector<Simu_or_mbp>> *sorm = nullptr;
	uint32_t k0 = 0, k1 = 0, stream = 0;
	unsigned sett = 0, c = 0, tr = 0, dp = 0;
	unsigned narea = 0, ntrans = 0, ndp = 0, ndiv = 0;
	unsigned long long ncalls = 0;
	void advance() {
		if (++dp < ndp) return;
		dp = 0;
		if (++tr < ntrans) return;
		tr = 0;
		if (++c < narea) return;
		c = 0; sett++;
	}
};
Replay g_replay;
}  // namespace

extern "C" int __real__Z14poisson_sampled(double lam);
extern "C" unsigned int __real__Z15binomial_sampledj(double p, unsigned int n);
extern "C" double __real__Z3ranv();

namespace {
// Kind of draw Mbp::mbp makes for the cell under the cursor (src/mbp.cc:284-305):
// 0 none, 1 Poisson(m'), 2 Poisson(m' - m), 3 Binomial(n, m'/m).
int mbp_kind(const Replay &r)
{
	const double mp = r.st->transmean[r.sett][r.c][r.tr][r.dp];
	if (mp == 0) return 0;
	if ((*r.sorm)[r.sett][r.c] == SIMU) return 1;
	const double mi = r.ini->transmean[r.sett][r.c][r.tr][r.dp];
	if (mp > mi) return 2;
	if (mp == mi) return 0;
	return 3;
}

// Moves the cursor to the next cell that draws; returns its kind.
int mbp_seek(Replay &r)
{
	while (true) {
		if (r.sett >= r.ndiv) { fprintf(stderr, "replay: cursor ran past the last step\n"); abort(); }
		const int k = mbp_kind(r);
		if (k) return k;
		r.advance();
	}
}
}  // namespace

// ran() (src/utils.cc:50-69) answered from the keyed stream while a bootstrap
// runs: the k-th call of section sec takes word 0 of
// Philox({k, sec, stream, RESAMPLE<<24}) as u = (w + 1/2) 2^-32.
namespace {
struct RanReplay {
	bool active = false;
	uint32_t k0 = 0, k1 = 0, stream = 0, sec = 0, k = 0;
};
RanReplay g_ran;
}  // namespace

extern "C" double __wrap__Z3ranv()
{
	RanReplay &r = g_ran;
	if (!r.active) return __real__Z3ranv();
	beep_u32x4 c = {{r.k, r.sec, r.stream, BEEP_PURPOSE_RESAMPLE << 24}};
	beep_u32x4 o = beep_philox4x32_10(c, r.k0, r.k1);
	r.k++;
	return beep_u01(o.v[0]);
}

// Answers the reference's k-th poisson_sample(mean) call of a simulate(ti,tf)
// with the keyed draw of the (sett, c, tr, dp) cell that call belongs to.  The
// cell is found by walking transmean[sett][c][tr][dp] in the reference's loop
// order (src/state.cc:608-631), skipping cells whose mean is 0 (no call).
extern "C" int __wrap__Z14poisson_sampled(double lam)
{
	Replay &r = g_replay;
	if (!r.active) return __real__Z14poisson_sampled(lam);
	if (r.mbp) {
		const int kind = mbp_seek(r);
		const double mp = r.st->transmean[r.sett][r.c][r.tr][r.dp];
		const double want = kind == 1 ? mp : mp - r.ini->transmean[r.sett][r.c][r.tr][r.dp];
		if (kind == 3 || memcmp(&want, &lam, sizeof lam) != 0) {
			fprintf(stderr, "replay: MBP Poisson mismatch at sett=%u c=%u tr=%u dp=%u (kind %d): %.17g vs %.17g\n",
			        r.sett, r.c, r.tr, r.dp, kind, want, lam);
			abort();
		}
		int v = beep_poisson_ref(lam, r.k0, r.k1, r.c * r.ndp + r.dp, r.tr, r.sett, r.stream);
		if (v < 0) { fprintf(stderr, "replay: rejection sampler gave up\n"); abort(); }
		r.ncalls++;
		r.advance();
		return v;
	}
	while (true) {
		if (r.sett >= r.ndiv) { fprintf(stderr, "replay: cursor ran past the last step\n"); abort(); }
		double m = r.st->transmean[r.sett][r.c][r.tr][r.dp];
		if (m != 0) break;
		r.advance();
	}
	double m = r.st->transmean[r.sett][r.c][r.tr][r.dp];
	if (memcmp(&m, &lam, sizeof m) != 0) {
		fprintf(stderr, "replay: mean mismatch at sett=%u c=%u tr=%u dp=%u: %.17g vs %.17g\n",
		        r.sett, r.c, r.tr, r.dp, m, lam);
		abort();
	}
	int v = beep_poisson_ref(lam, r.k0, r.k1, r.c * r.ndp + r.dp, r.tr, r.sett, r.stream);
	if (v < 0) { fprintf(stderr, "replay: rejection sampler gave up\n"); abort(); }
	r.ncalls++;
	r.advance();
	return v;
}

// binomial_sample(p, n) (src/utils.cc:174-180), called by Mbp::mbp when the
// proposed mean is below the initial one: answered with the keyed thinning
// draw of the cell under the cursor.
extern "C" unsigned int __wrap__Z15binomial_sampledj(double p, unsigned int n)
{
	Replay &r = g_replay;
	if (!r.active || !r.mbp) return __real__Z15binomial_sampledj(p, n);
	const int kind = mbp_seek(r);
	const double mp = r.st->transmean[r.sett][r.c][r.tr][r.dp], mi = r.ini->transmean[r.sett][r.c][r.tr][r.dp];
	const double want = mp / mi;
	const int ni = (int)r.ini->transnum[r.sett][r.c][r.tr][r.dp];
	if (kind != 3 || memcmp(&want, &p, sizeof p) != 0 || (unsigned int)ni != n) {
		fprintf(stderr, "replay: MBP binomial mismatch at sett=%u c=%u tr=%u dp=%u (kind %d): p %.17g vs %.17g, n %d vs %u\n",
		        r.sett, r.c, r.tr, r.dp, kind, want, p, ni, n);
		abort();
	}
	int v = beep_binomial_ref(p, (int32_t)n, r.k0, r.k1, r.c * r.ndp + r.dp, r.tr, r.sett, r.stream);
	if (v < 0) { fprintf(stderr, "replay: binomial rejection sampler gave up\n"); abort(); }
	r.ncalls++;
	r.advance();
	return (unsigned int)v;
}

// ---- bundle writer -------------------------------------------------------

namespace {
struct Bundle {
	FILE *f = nullptr;
	void open(const std::string &fn) {
		f = fopen(fn.c_str(), "wb");
		if (!f) { fprintf(stderr, "cannot open %s\n", fn.c_str()); exit(1); }
		fwrite("BEEPBND1", 1, 8, f);
	}
	void rec(const std::string &name, char type, const std::vector<uint64_t> &dims, const void *data, size_t esz) {
		uint32_t nl = (uint32_t)name.size();
		fwrite(&nl, 4, 1, f); fwrite(name.data(), 1, nl, f);
		fwrite(&type, 1, 1, f);
		uint32_t nd = (uint32_t)dims.size(); fwrite(&nd, 4, 1, f);
		size_t n = 1;
		for (auto d : dims) { fwrite(&d, 8, 1, f); n *= d; }
		if (n) fwrite(data, esz, n, f);
	}
	void d(const std::string &n, const std::vector<double> &v, std::vector<uint64_t> dims = {}) {
		if (dims.empty()) dims = {v.size()};
		rec(n, 'd', dims, v.data(), 8);
	}
	void i(const std::string &n, const std::vector<int32_t> &v, std::vector<uint64_t> dims = {}) {
		if (dims.empty()) dims = {v.size()};
		rec(n, 'i', dims, v.data(), 4);
	}
	void scalar_d(const std::string &n, double v) { d(n, std::vector<double>{v}); }
	void scalar_i(const std::string &n, int32_t v) { i(n, std::vector<int32_t>{v}); }
	void close() { if (f) fclose(f); f = nullptr; }
};

std::vector<std::vector<double>> read_theta(const std::string &fn)
{
	std::vector<std::vector<double>> out;
	std::ifstream in(fn);
	std::string line;
	while (std::getline(in, line)) {
		if (line.empty()) continue;
		std::vector<double> row;
		std::stringstream ss(line);
		std::string tok;
		while (std::getline(ss, tok, ',')) row.push_back(strtod(tok.c_str(), nullptr));
		out.push_back(row);
	}
	return out;
}
}  // namespace

int main(int argc, char **argv)
{
	std::map<std::string, std::string> opt;
	int split = argc;
	for (int k = 1; k < argc; k++) {
		if (std::string(argv[k]) == "--") { split = k; break; }
		std::string s = argv[k];
		auto e = s.find('=');
		if (e == std::string::npos) { fprintf(stderr, "bad option %s\n", argv[k]); return 2; }
		opt[s.substr(0, e)] = s.substr(e + 1);
	}
	if (!opt.count("out")) { fprintf(stderr, "out= is required\n"); return 2; }
	int npart = opt.count("npart") ? atoi(opt["npart"].c_str()) : 4;
	int ntraj = opt.count("ntraj") ? atoi(opt["ntraj"].c_str()) : 1;
	uint64_t seed = opt.count("seed") ? strtoull(opt["seed"].c_str(), nullptr, 0) : 12345;
	bool pf = opt.count("pf") && opt["pf"] == "1";

	std::vector<char *> bargv;
	bargv.push_back(argv[0]);
	for (int k = split + 1; k < argc; k++) bargv.push_back(argv[k]);
	int bargc = (int)bargv.size();

	timersinit();
	MPI_Init(&bargc, nullptr);
	Inputs inputs(bargc, bargv.data());
	Details details(inputs);
	Mpi mpi(details);
	Data data(inputs, details, mpi);
	Model model(inputs, details, data, mpi);
	sran(mpi.core * 10000 + inputs.find_integer("seed", 0) + 100);
	ObservationModel obsmodel(details, data, model);

	const unsigned A = data.narea, G = data.nage, DP = data.ndemocatpos, NS = data.nstrain;
	const unsigned C = model.comp.size(), T = model.trans.size(), S = details.ndivision;
	const unsigned DPS = data.ndemocatpos_per_strain;

	std::vector<std::vector<double>> thetas;
	if (opt.count("theta")) thetas = read_theta(opt["theta"]);
	else thetas.push_back(model.simulated_values());
	for (auto &th : thetas) {
		if (th.size() != model.param.size()) { fprintf(stderr, "theta has %zu values, model has %zu parameters\n", th.size(), model.param.size()); return 2; }
	}
	int ngroup = (int)thetas.size();

	Bundle B;
	B.open(opt["out"]);

	// ---- parameter-independent model (beep_model_desc) ----
	B.i("dims", {(int32_t)A, (int32_t)G, (int32_t)DP, (int32_t)NS, (int32_t)C, (int32_t)T, (int32_t)S,
	             (int32_t)details.period, (int32_t)details.division_per_time});
	B.scalar_d("dt", double(details.period) / details.ndivision);
	B.scalar_d("popsize", (double)data.popsize);
	// the model through the binding a BEEP maintainer adds (beep_gb300/binding): the bundle
	// holds exactly what it packs for beep_model_create
	const beep_binding::ModelPack mp(details, data, model);
	B.i("trans_from", mp.trans_from); B.i("trans_to", mp.trans_to);
	B.scalar_i("infection_trans", mp.desc.infection_trans);
	B.i("democatpos_age", mp.democatpos_age);
	B.d("M_diag", mp.M_diag); B.i("M_rowptr", mp.M_rowptr); B.i("M_to", mp.M_to); B.d("M_val", mp.M_val);
	B.d("M_factor", mp.M_factor);
	B.d("pop_init", mp.pop_init, {A, C, DP});
	B.i("obs_sett_i", mp.obs_sett_i); B.i("obs_sett_f", mp.obs_sett_f); B.i("obs_value_kind", mp.obs_value_kind);
	B.d("obs_value", mp.obs_value); B.i("obs_model", mp.obs_model); B.d("obs_sd", mp.obs_sd);
	B.d("obs_shape", mp.obs_shape); B.d("obs_threshold", mp.obs_threshold); B.d("obs_factor", mp.obs_factor);
	B.i("obs_factor_spline", mp.obs_factor_spline); B.i("obs_cell_ptr", mp.obs_cell_ptr); B.i("obs_cells", mp.obs_cells);
	// demographic changes (populations become fractional: trajectories are written in FP64)
	const bool pop64 = !data.democat_change.empty();
	if (pop64) {
		B.i("dcc_nval", mp.dcc_nval); B.i("dcc_area_ptr", mp.dcc_area_ptr); B.i("dcc_area", mp.dcc_area);
		B.i("dcc_dp_ptr", mp.dcc_dp_ptr); B.i("dcc_dp", mp.dcc_dp); B.d("dcc_frac", mp.dcc_frac);
	}
	if (pf) {
		std::vector<int32_t> sti, stf;
		for (unsigned s = 0; s < obsmodel.nsection; s++) { sti.push_back(obsmodel.section_ti[s]); stf.push_back(obsmodel.section_tf[s]); }
		B.i("section_ti", sti); B.i("section_tf", stf);
	}

	// ---- per parameter set: tables from set_param, then the particles ----
	g_replay.k0 = (uint32_t)seed; g_replay.k1 = (uint32_t)(seed >> 32);
	g_replay.narea = A; g_replay.ntrans = T; g_replay.ndp = DP; g_replay.ndiv = S;
	B.i("seed_words", {(int32_t)g_replay.k0, (int32_t)g_replay.k1});
	B.scalar_i("ngroup", ngroup);
	{
		std::vector<int32_t> names;
		for (const auto &par : model.param) {
			for (char ch : par.name) names.push_back((int32_t)(unsigned char)ch);
			names.push_back('\n');
		}
		B.i("param_names", names);
	}
	B.scalar_i("npart", npart);
	B.scalar_i("ntraj", ntraj);

	// the tables State::set_param produced for parameter set theta (beep_param_tables), and in
	// prediction mode the model modifications' multipliers (ModelMod, src/model.cc:1446-1585)
	auto dump_tables = [&](const std::string &gp, const State &state, const std::vector<double> &theta) {
		const beep_binding::TablePack tp(mp, details, data, model, state, theta);
		B.d(gp + "transrate", tp.transrate, {T, DP});
		B.d(gp + "susceptibility", tp.susceptibility);
		B.d(gp + "infectivity", tp.infectivity);
		B.d(gp + "beta_rows", tp.beta_rows, {(uint64_t)tp.tables.nbeta_row, S});
		B.i(gp + "beta_row_of", tp.beta_row_of, {NS, A});
		B.d(gp + "areafactor", tp.areafactor, {details.period, A});
		B.d(gp + "Ntime", tp.Ntime, {S, G, G});
		B.d(gp + "geo_spline", tp.geo_spline);
		B.d(gp + "efoi_spline", tp.efoi_spline, {(uint64_t)tp.tables.nefoi, S});
		B.d(gp + "efoi_agedist", tp.efoi_agedist, {(uint64_t)tp.tables.nefoi, G});
		B.i(gp + "efoi_ref", tp.efoi_ref, {NS, A});
		B.d(gp + "obs_spline", tp.obs_spline, {(uint64_t)tp.tables.nobs_spline, S});
		if (!tp.efoi_mult.empty()) {
			B.d(gp + "efoi_mult", tp.efoi_mult, {S, A, NS});
			B.d(gp + "transmean_mult", tp.transmean_mult, {S, A, T, DP});
		}
	};

	// the priors through the binding, and the reference's own Model::prior / inbounds of
	// every parameter row and of probe rows (each parameter in turn moved below its
	// lower or above its upper uniform bound, or scaled by 1.1)
	{
		const beep_binding::PriorPack pp(details, model);
		const uint64_t np = pp.type.size();
		B.i("prior.type", pp.type); B.d("prior.val1", pp.val1); B.d("prior.val2", pp.val2);
		B.i("prior.val1_param", pp.val1_param); B.i("prior.val2_param", pp.val2_param);
		B.i("prior.gt_ptr", pp.gt_ptr); B.i("prior.gt_param", pp.gt_param);
		B.i("prior.lt_ptr", pp.lt_ptr); B.i("prior.lt_param", pp.lt_param);
		B.i("prior.dir_ptr", pp.dir_ptr); B.i("prior.dir_param", pp.dir_param); B.d("prior.dir_frac", pp.dir_frac);
		B.i("prior.smooth_kind", pp.smooth_kind); B.i("prior.smooth_par1", pp.smooth_par1);
		B.i("prior.smooth_par2", pp.smooth_par2); B.d("prior.smooth_mult1", pp.smooth_mult1);
		B.d("prior.smooth_mult2", pp.smooth_mult2); B.d("prior.smooth_value", pp.smooth_value);
		B.scalar_i("prior.ml_mode", pp.spec.ml_mode);
		std::vector<double> rows, Pr;
		std::vector<int32_t> inb;
		for (const auto &th : thetas) {
			std::vector<std::vector<double>> probes{th};
			for (unsigned k = 0; k < np; k++) {
				auto t2 = th;
				if (model.param[k].priortype == UNIFORM_PRIOR) {
					auto t3 = th;
					t2[k] = model.param[k].val1 - 0.5;
					t3[k] = model.param[k].val2 + 0.5;
					probes.push_back(t3);
				} else {
					t2[k] = th[k] * 1.1;
				}
				probes.push_back(t2);
			}
			for (const auto &p : probes) {
				rows.insert(rows.end(), p.begin(), p.end());
				const bool ok = model.inbounds(p);
				inb.push_back(ok ? 1 : 0);
				Pr.push_back(ok ? model.prior(p) : 0.0);
			}
		}
		B.d("prior.theta", rows, {(uint64_t)inb.size(), np});
		B.i("prior.inbounds", inb);
		B.d("prior.logprior", Pr);
	}

	for (int gidx = 0; gidx < ngroup; gidx++) {
		std::string gp = "g" + std::to_string(gidx) + ".";
		B.d(gp + "theta", thetas[gidx]);
		State state(details, data, model, obsmodel);
		state.set_param(thetas[gidx]);
		dump_tables(gp, state, thetas[gidx]);

		std::vector<double> Lfull(npart), Lsec;
		std::vector<int32_t> tnum, popt;
		std::vector<double> chk, popd;
		for (int p = 0; p < npart; p++) {
			uint32_t stream = (uint32_t)(gidx * npart + p);
			g_replay.st = &state; g_replay.stream = stream;
			g_replay.sett = 0; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
			g_replay.active = true;
			if (!pf) {
				state.simulate(thetas[gidx]);
				Lfull[p] = obsmodel.calculate(&state);
			} else {
				state.set_param(thetas[gidx]);
				for (unsigned sec = 0; sec < obsmodel.nsection; sec++) {
					unsigned ti = obsmodel.section_ti[sec], tf2 = obsmodel.section_tf[sec];
					g_replay.sett = ti; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
					state.simulate(ti, tf2);
					Lsec.push_back(obsmodel.calculate_section(&state, sec));
				}
				Lfull[p] = obsmodel.calculate(&state);
			}
			g_replay.active = false;
			// checksums over the whole trajectory (exact integer sums, weighted)
			double s1 = 0, s2 = 0, s3 = 0, s4 = 0;
			for (unsigned s = 0; s < S; s++)
				for (unsigned c = 0; c < A; c++) {
					for (unsigned tr = 0; tr < T; tr++)
						for (unsigned dp = 0; dp < DP; dp++) {
							double v = state.transnum[s][c][tr][dp];
							s1 += v; s2 += v * (double)(1 + ((s * 131 + c * 31 + tr * 7 + dp) % 1009));
						}
					for (unsigned co = 0; co < C; co++)
						for (unsigned dp = 0; dp < DP; dp++) {
							double v = state.pop[s][c][co][dp];
							s3 += v; s4 += v * (double)(1 + ((s * 131 + c * 31 + co * 7 + dp) % 1009));
						}
				}
			chk.insert(chk.end(), {s1, s2, s3, s4});
			if (p < ntraj) {
				for (unsigned s = 0; s < S; s++)
					for (unsigned c = 0; c < A; c++) {
						for (unsigned tr = 0; tr < T; tr++)
							for (unsigned dp = 0; dp < DP; dp++) tnum.push_back((int32_t)state.transnum[s][c][tr][dp]);
						for (unsigned co = 0; co < C; co++)
							for (unsigned dp = 0; dp < DP; dp++) {
								popt.push_back((int32_t)state.pop[s][c][co][dp]);
								popd.push_back(state.pop[s][c][co][dp]);
							}
					}
			}
		}
		if (pf && opt.count("pfn")) {
			// PMCMC::obs_prob (src/pmcmc.cc:180-207) driven section by section with
			// the reference's own end_sec_swap and bootstrap; particle slot p draws
			// from stream p, the resampling uniforms from stream `pfstream`.
			const int NP = atoi(opt["pfn"].c_str());
			const uint32_t pfstream = opt.count("pfstream") ? (uint32_t)strtoul(opt["pfstream"].c_str(), nullptr, 0) : 0xABCDu;
			Output output(details, data, model, inputs, obsmodel, mpi);
			PMCMC pm(details, data, model, inputs, output, obsmodel, mpi);
			if ((int)pm.Ntot != NP) { fprintf(stderr, "nparticle must equal pfn\n"); return 2; }
			pm.particle.clear();
			for (int p2 = 0; p2 < NP; p2++) pm.particle.push_back(State(details, data, model, obsmodel));
			for (int p2 = 0; p2 < NP; p2++) pm.particle[p2].set_param(thetas[gidx]);
			std::vector<double> L(NP), Lsecs, obp;
			std::vector<int32_t> anc;
			double obprob = 0.0;
			for (unsigned sec = 0; sec < obsmodel.nsection; sec++) {
				const unsigned ti = obsmodel.section_ti[sec], tf2 = obsmodel.section_tf[sec];
				if (sec > 0) mpi.end_sec_swap(pm.particle, ti, pm.backpart[sec], pm.buffersize);
				for (int p2 = 0; p2 < NP; p2++) {
					g_replay.st = &pm.particle[p2]; g_replay.stream = (uint32_t)p2;
					g_replay.sett = ti; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
					g_replay.active = true;
					pm.particle[p2].simulate(ti, tf2);
					g_replay.active = false;
					L[p2] = obsmodel.calculate_section(&pm.particle[p2], sec);
				}
				Lsecs.insert(Lsecs.end(), L.begin(), L.end());
				g_ran.active = true; g_ran.k0 = g_replay.k0; g_ran.k1 = g_replay.k1;
				g_ran.stream = pfstream; g_ran.sec = sec; g_ran.k = 0;
				const double ob = pm.bootstrap(sec, L);
				g_ran.active = false;
				obprob += ob;
				obp.push_back(ob);
				for (int p2 = 0; p2 < NP; p2++) anc.push_back((int32_t)pm.backpart[sec + 1][p2]);
			}
			// the sampled lineage (Mpi::particle_sample, src/mpi.cc:331-389) and, when
			// sampledir= is given, its sample files (Mpi::gather_samples -> State::save,
			// src/mpi.cc:677-720, src/state.cc:709-739)
			{
				Particle part = mpi.particle_sample(0, pm.backpart, pm.particle, obsmodel);
				std::vector<int32_t> lin;
				for (unsigned s = 0; s < S; s++)
					for (unsigned c = 0; c < A; c++)
						for (unsigned tr = 0; tr < T; tr++)
							for (unsigned dp = 0; dp < DP; dp++) lin.push_back((int32_t)part.transnum[s][c][tr][dp]);
				B.i(gp + "pf.lineage_transnum", lin, {S, A, T, DP});
				B.scalar_d(gp + "pf.lineage_EF", part.EF);
				if (opt.count("sampledir")) {           // Mpi::gather_samples, src/mpi.cc:677-720
					std::vector<ParamSample> psamp;
					std::vector<Sample> opsamp;
					std::vector<Particle> parts{part};
					State st(details, data, model, obsmodel);
					mpi.gather_samples(psamp, opsamp, parts, st, opt["sampledir"] + "/");
				}
			}
			B.scalar_d(gp + "pf.obprob", obprob);
			B.d(gp + "pf.obprob_section", obp);
			B.d(gp + "pf.L_section", Lsecs, {obsmodel.nsection, (uint64_t)NP});
			B.i(gp + "pf.ancestors", anc, {obsmodel.nsection, (uint64_t)NP});
			B.scalar_d(gp + "pf.invT", pm.invT);
			B.i(gp + "pf.stream", {(int32_t)pfstream});
		}
		B.d(gp + "L", Lfull);
		if (pf) B.d(gp + "L_section", Lsec, {(uint64_t)npart, obsmodel.nsection});
		B.d(gp + "checksum", chk, {(uint64_t)npart, 4});
		int nt = std::min(ntraj, npart);
		B.i(gp + "transnum", tnum, {(uint64_t)nt, S, A, T, DP});
		if (pop64) B.d(gp + "pop", popd, {(uint64_t)nt, S, A, C, DP});
		else B.i(gp + "pop", popt, {(uint64_t)nt, S, A, C, DP});
	}
	if (opt.count("pred")) {
		// Prediction (Simulate::model_modification, src/simulate.cc:142-165): each posterior
		// sample <pred>/sample<k> is loaded (State::load, src/state.cc:743-808) and simulated
		// from the modifications' start to the end (State::simulate(ti, tf)) under the
		// model's modifications, on stream 7000 + k.
		const std::string dir = opt["pred"] + "/";
		const int K = opt.count("predn") ? atoi(opt["predn"].c_str()) : 1;
		const unsigned ti = model.modelmod.pred_start * details.division_per_time;
		B.scalar_i("pred.n", K);
		B.scalar_i("pred.ti", (int32_t)ti);
		State st(details, data, model, obsmodel);
		for (int k = 0; k < K; k++) {
			const std::string pk = "pred" + std::to_string(k) + ".";
			st.load(dir + "sample" + std::to_string(k), S);
			B.d(pk + "theta", st.paramval);
			dump_tables(pk, st, st.paramval);
			std::vector<int32_t> p0, tn, p1;
			for (unsigned c = 0; c < A; c++)
				for (unsigned co = 0; co < C; co++)
					for (unsigned dp = 0; dp < DP; dp++) p0.push_back((int32_t)st.pop[ti][c][co][dp]);
			g_replay.mbp = false; g_replay.st = &st; g_replay.stream = 7000u + k;
			g_replay.sett = ti; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
			g_replay.active = true;
			st.simulate(ti, S);
			g_replay.active = false;
			for (unsigned s2 = ti; s2 < S; s2++)
				for (unsigned c = 0; c < A; c++)
					for (unsigned tr = 0; tr < T; tr++)
						for (unsigned dp = 0; dp < DP; dp++) tn.push_back((int32_t)st.transnum[s2][c][tr][dp]);
			// the populations after the last step (State::simulate updates them only up to
			// the last step's start): update_pop's arithmetic on the last step's counts
			for (unsigned c = 0; c < A; c++) {
				auto pe = st.pop[S - 1][c];
				for (unsigned tr = 0; tr < T; tr++)
					for (unsigned dp = 0; dp < DP; dp++) {
						const double num = st.transnum[S - 1][c][tr][dp];
						if (num != 0) { pe[model.trans[tr].from][dp] -= num; pe[model.trans[tr].to][dp] += num; }
					}
				for (unsigned co = 0; co < C; co++)
					for (unsigned dp = 0; dp < DP; dp++) p1.push_back((int32_t)pe[co][dp]);
			}
			B.i(pk + "pop_ti", p0, {A, C, DP});
			B.i(pk + "transnum", tn, {(uint64_t)(S - ti), A, T, DP});
			B.i(pk + "pop_end", p1, {A, C, DP});
			B.i(pk + "stream", {(int32_t)(7000 + k)});
		}
	}
	if (opt.count("mbp")) {
		// MBP chains (src/mbp.cc:252-361,460-491, src/state.cc:812-826).  Chain k
		// starts from State::simulate(theta[2k]) on stream 1000+k; its proposal is
		// Mbp::mbp(theta[2k+1]) on stream 2000+100v+k in three variants v:
		// 0 INF_DIF_UPDATE, 1 INF_UPDATE, 2 INF_DIF_UPDATE with SIMU cells
		// (steps [S/4, S/2), areas with (c + sett + k) even).
		const int NC = atoi(opt["mbp"].c_str());
		if ((int)thetas.size() < 2 * NC) { fprintf(stderr, "mbp=%d needs %d parameter rows\n", NC, 2 * NC); return 2; }
		Output output(details, data, model, inputs, obsmodel, mpi);
		Mbp mb(INVT, details, data, model, obsmodel, output, mpi);
		mb.invT = 1.0;
		const InfUpdate iu[3] = {INF_DIF_UPDATE, INF_UPDATE, INF_DIF_UPDATE};
		B.scalar_i("mbp.nchain", NC);
		for (int v = 0; v < 3; v++) {
			std::string vp = "mbp" + std::to_string(v) + ".";
			std::vector<double> Li_, Lp_, Lii, Lif, EFi, EFp, Pri, Prp, al, chk;
			std::vector<int32_t> simu((size_t)NC * S * A, 0), tni, tnp, si, sp;
			for (int k = 0; k < NC; k++) {
				State *ini = mb.initial;
				g_replay.mbp = false; g_replay.st = ini; g_replay.stream = 1000u + k;
				g_replay.sett = 0; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
				g_replay.active = true;
				ini->simulate(thetas[2 * k]);
				g_replay.active = false;
				Li_.push_back(obsmodel.calculate(ini)); EFi.push_back(ini->EF); Pri.push_back(ini->Pr);
				Lii.push_back(ini->likelihood());
				mb.copy_initial_to_propse();                      // parameter_proposal on the fixed state
				mb.propose->set_param(thetas[2 * k + 1]);
				for (unsigned sett = 0; sett < S; sett++)
					for (unsigned c = 0; c < A; c++) mb.propose->set_transmean(sett, c);
				Lif.push_back(mb.propose->likelihood());
				mb.simu_or_mbp_reset();
				if (v == 2)
					for (unsigned sett = S / 4; sett < S / 2; sett++)
						for (unsigned c = 0; c < A; c++)
							if ((c + sett + k) % 2 == 0) { mb.simu_or_mbp[sett][c] = SIMU; simu[((size_t)k * S + sett) * A + c] = 1; }
				g_replay.mbp = true; g_replay.st = mb.propose; g_replay.ini = mb.initial; g_replay.sorm = &mb.simu_or_mbp;
				g_replay.stream = 2000u + 100u * v + k;
				g_replay.sett = 0; g_replay.c = 0; g_replay.tr = 0; g_replay.dp = 0;
				g_replay.active = true;
				Status ok = mb.mbp(thetas[2 * k + 1], iu[v]);
				g_replay.active = false; g_replay.mbp = false;
				if (ok != SUCCESS) { fprintf(stderr, "mbp: proposal %d outside the prior bounds\n", k); return 2; }
				al.push_back(mb.get_al());                        // sets the proposal's EF and Pr
				Lp_.push_back(obsmodel.calculate(mb.propose)); EFp.push_back(mb.propose->EF); Prp.push_back(mb.propose->Pr);
				si.push_back((int32_t)(1000u + k)); sp.push_back((int32_t)(2000u + 100u * v + k));
				for (const State *x : {(const State *)mb.initial, (const State *)mb.propose}) {
					double s1 = 0, s2 = 0;
					for (unsigned s = 0; s < S; s++)
						for (unsigned c = 0; c < A; c++)
							for (unsigned tr = 0; tr < T; tr++)
								for (unsigned dp = 0; dp < DP; dp++) {
									double val = x->transnum[s][c][tr][dp];
									s1 += val; s2 += val * (double)(1 + ((s * 131 + c * 31 + tr * 7 + dp) % 1009));
								}
					chk.push_back(s1); chk.push_back(s2);
				}
				if (k < ntraj)
					for (unsigned s = 0; s < S; s++)
						for (unsigned c = 0; c < A; c++)
							for (unsigned tr = 0; tr < T; tr++)
								for (unsigned dp = 0; dp < DP; dp++) {
									tni.push_back((int32_t)mb.initial->transnum[s][c][tr][dp]);
									tnp.push_back((int32_t)mb.propose->transnum[s][c][tr][dp]);
								}
			}
			B.scalar_i(vp + "inf_update", (int32_t)iu[v]);
			B.i(vp + "simu", simu, {(uint64_t)NC, S, A});
			B.i(vp + "stream_init", si); B.i(vp + "stream_prop", sp);
			B.d(vp + "L_init", Li_); B.d(vp + "L_prop", Lp_); B.d(vp + "Li_init", Lii); B.d(vp + "Li_fixed", Lif);
			B.d(vp + "EF_init", EFi); B.d(vp + "EF_prop", EFp); B.d(vp + "Pr_init", Pri); B.d(vp + "Pr_prop", Prp);
			B.d(vp + "al", al);
			B.d(vp + "checksum", chk, {(uint64_t)NC, 2, 2});
			const int nt = std::min(ntraj, NC);
			B.i(vp + "transnum_init", tni, {(uint64_t)nt, S, A, T, DP});
			B.i(vp + "transnum_prop", tnp, {(uint64_t)nt, S, A, T, DP});
		}
	}
	if (opt.count("abcw")) {
		const int NN = atoi(opt["abcw"].c_str()), K = atoi(opt["abck"].c_str());
		if (K < 2 || NN < 1 || (int)thetas.size() < K + NN) {
			fprintf(stderr, "abcw=%d abck=%d needs %d parameter rows\n", NN, K, K + NN);
			return 2;
		}
		Output output(details, data, model, inputs, obsmodel, mpi);
		ABCSMC abc(details, data, model, inputs, output, obsmodel, mpi);
		Generation gl;
		for (int j = 0; j < K; j++) {
			ParamSample ps;
			ps.run = 0; ps.EF = 0; ps.paramval = thetas[j];
			gl.param_samp.push_back(ps);
			gl.w.push_back(0.5 + 0.1 * (j % 7));
		}
		MVN mvn("ABCSMC", model.param_not_fixed, abc.propsize, ALL_PARAM, MULTIPLE);
		mvn.setup(gl.param_samp, gl.w);
		Generation gn;
		std::vector<double> lp, tn, tl;
		for (int i = 0; i < NN; i++) {
			const auto &th = thetas[K + i];
			gn.w.push_back(abc.calculate_particle_weight(th, gl, mvn));
			ParamSample ps;
			ps.run = 0; ps.EF = 0; ps.paramval = th;
			gn.param_samp.push_back(ps);                     // normalise_particle_weights counts these
			lp.push_back(model.prior(th));
			for (auto v : mvn.var) tn.push_back(th[v]);
		}
		for (int j = 0; j < K; j++)
			for (auto v : mvn.var) tl.push_back(thetas[j][v]);
		const std::vector<double> w_raw = gn.w;
		abc.normalise_particle_weights(gn);
		std::vector<double> inv;
		for (auto &row : mvn.inv_M) inv.insert(inv.end(), row.begin(), row.end());
		const uint64_t nv = mvn.var.size();
		B.scalar_d("abc.size", mvn.size);
		B.d("abc.theta_new", tn, {(uint64_t)NN, nv}); B.d("abc.logprior_new", lp);
		B.d("abc.theta_last", tl, {(uint64_t)K, nv}); B.d("abc.w_last", gl.w);
		B.d("abc.inv_cov", inv, {nv, nv});
		B.d("abc.w", w_raw); B.d("abc.w_norm", gn.w);
	}
	B.close();
	fprintf(stderr, "ref_harness: %d groups x %d particles, %llu keyed draws\n", ngroup, npart, g_replay.ncalls);
	return 0;
}
