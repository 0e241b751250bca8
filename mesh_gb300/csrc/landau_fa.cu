// Host side of Fourier-accelerated Landau gauge fixing: the workspace object,
// the step, the run loop with the overrelaxation fallback, and the
// per-momentum response probe (training data of the learned multiplier).
#include "landau_fa.cuh"

#include <cmath>
#include <limits>
#include <vector>

using namespace meshgb;

namespace {

struct FaTable
{
	void (*links)(Field const &U, Field const &g, double *A, RedSlot func);
	void (*div)(Field const &U, double const *A, float2 *buf, RedSlot theta);
	void (*update)(Field const &U, float2 const *buf, Field const &gin, double *gout);
};

template <int GRP, int ND> struct FaOps
{
	static void links(Field const &U, Field const &g, double *A, RedSlot func)
	{
		auto &c = *U.ctx;
		int64_t n = int64_t(ND) * U.geom.V;
		k_fa_links<GRP, double, ND><<<grid_for(c, n, 256), 256, 0, c.stream>>>(
		    U.geom, static_cast<double const *>(U.d), static_cast<double const *>(g.d), A, func);
		MESH_LAUNCH_CHECK();
	}
	static void div(Field const &U, double const *A, float2 *buf, RedSlot theta)
	{
		auto &c = *U.ctx;
		unsigned b = grid_for(c, U.geom.V, 256, 4);
		k_fa_div<GRP, double, ND><<<b, 256, 0, c.stream>>>(U.geom, A, buf, theta);
		MESH_LAUNCH_CHECK();
	}
	static void update(Field const &U, float2 const *buf, Field const &gin, double *gout)
	{
		auto &c = *U.ctx;
		k_fa_update<GRP, double, ND><<<grid_for(c, U.geom.V, 256), 256, 0, c.stream>>>(
		    U.geom, buf, static_cast<double const *>(gin.d), gout, 1.0 / double(U.geom.V));
		MESH_LAUNCH_CHECK();
	}
	static FaTable const *table()
	{
		static const FaTable t = {links, div, update};
		return &t;
	}
};

FaTable const *fa_table(int grp, int nd)
{
	switch (grp * 10 + nd)
	{
	case 12:
		return FaOps<U1, 2>::table();
	case 13:
		return FaOps<U1, 3>::table();
	case 14:
		return FaOps<U1, 4>::table();
	case 22:
		return FaOps<SU2, 2>::table();
	case 23:
		return FaOps<SU2, 3>::table();
	case 24:
		return FaOps<SU2, 4>::table();
	case 32:
		return FaOps<SU3, 2>::table();
	case 33:
		return FaOps<SU3, 3>::table();
	case 34:
		return FaOps<SU3, 4>::table();
	default:
		return nullptr;
	}
}

template <class F> int fa_api(F &&f) { return api_call(f); }
} // namespace

struct mesh_landau_fa_s
{
	Field const *U = nullptr;
	Context *ctx = nullptr;
	FaTable const *tab = nullptr;
	int nf = 0;          // complex FFT fields
	double *A = nullptr; // nd x NA x V
	float2 *buf = nullptr, *buf_old = nullptr;
	double *g_trial = nullptr;
	// reduction scratch, two slots (0: theta, 1: the gauge functional):
	// partials, results, counters
	double *red = nullptr;
	double *res = nullptr;
	unsigned *cnt = nullptr;
	// accept a descent step when the gauge functional did not drop (instead
	// of when theta dropped)
	bool accept_functional = false;
	float *table = nullptr; // learned multiplier table (device)
	MomTables mt{};
	Multiplier mult{};
	std::vector<float> host_table;
	// learned multiplier: network parameters and feature buffer (device)
	float *mlp_params = nullptr, *mlp_x = nullptr;
	int mlp_width = 0, mlp_n = 256;
	bool mlp_bf16 = true;
	double mlp_beta = 6.0;
	bool learned = false;
	// probe accumulators
	double *shell = nullptr;
	int shell_bins = 0;

	RedSlot slot(int k = 0) { return {red + size_t(k) * kMaxRedBlocks, res + k, cnt + k}; }

	~mesh_landau_fa_s()
	{
		cudaFree(A);
		cudaFree(buf);
		cudaFree(buf_old);
		cudaFree(g_trial);
		cudaFree(red);
		cudaFree(res);
		cudaFree(cnt);
		cudaFree(table);
		cudaFree(shell);
		cudaFree(mlp_params);
		cudaFree(mlp_x);
	}

	// evaluate the network on the table grid for the current theta
	void refresh_learned(double th)
	{
		float lo = mult.lo, hi = mult.hi;
		float f1 = float(5.0 * (mlp_beta - 6.0));
		float f2 = float((std::log10(std::max(th, 1e-30)) + 7.0) / 5.0);
		k_fa_features<<<1, 256, 0, ctx->stream>>>(mlp_n, lo, hi, std::log(mt.p2max), f1, f2, mlp_x);
		MESH_LAUNCH_CHECK();
		mlp_forward_device(*ctx, mlp_n, mlp_x, mlp_params, mlp_width, mlp_bf16, table);
	}

	// theta of g; leaves Delta (FP32 complex) in buf when want_buf; with
	// `func`, also the sum of Re tr g(x) U_mu(x) g(x+mu)^+ over all links
	double theta(Field const &g, bool want_buf, double *func = nullptr)
	{
		tab->links(*U, g, A, func ? slot(1) : RedSlot{nullptr, nullptr, nullptr});
		tab->div(*U, A, want_buf ? buf : nullptr, slot(0));
		double v[2] = {0, 0};
		MESH_CUDA(cudaMemcpyAsync(v, res, sizeof(double) * (func ? 2 : 1), cudaMemcpyDeviceToHost, ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		if (func)
			*func = v[1];
		return v[0] / (double(U->nd) * double(U->geom.V));
	}

	// step on buf (Delta of g already there): gout = reunit(exp(-F^-1[m F Delta]/V) gin)
	void step_from_buf(Field const &gin, double *gout, Multiplier const &m, double th)
	{
		cudaStream_t s = ctx->stream;
		if (learned && m.mode == 1)
			refresh_learned(th);
		fft::fft_nd<-1>(buf, U->nd, U->dims, nf, ctx->num_sms, s);
		k_fa_scale<<<grid_for(*ctx, U->geom.V, 256), 256, 0, s>>>(buf, U->geom.V, nf, mt, m);
		MESH_LAUNCH_CHECK();
		fft::fft_nd<+1>(buf, U->nd, U->dims, nf, ctx->num_sms, s);
		tab->update(*U, buf, gin, gout);
	}
};

extern "C" {

int mesh_landau_fa_create(mesh_field Uh, mesh_landau_fa_s **out)
{
	if (!out)
		return MESH_ERR_ARG;
	*out = nullptr;
	auto *h = new mesh_landau_fa_s();
	int rc = fa_api([&] {
		require(Uh != nullptr, "null field");
		Field const &U = Uh->f;
		require(U.kind == MESH_GROUP && U.nstack == U.nd, "expected a gauge field");
		require(U.prec == MESH_F64, "Fourier-accelerated gauge fixing runs on FP64 links");
		for (int i = 0; i < U.nd; ++i)
			require(fft::supported_extent(U.dims[i]), "FFT extents must be one of 2,4,6,8,12,16,24,32");
		h->U = &U;
		h->ctx = U.ctx;
		h->tab = fa_table(U.group, U.nd);
		require(h->tab != nullptr, "unsupported group/dimension");
		int na = group_na(U.group);
		h->nf = (na + 1) / 2;
		int64_t V = U.geom.V;
		DeviceGuard dg(U.ctx->device);
		MESH_CUDA(cudaMalloc(&h->A, sizeof(double) * size_t(U.nd) * na * V));
		MESH_CUDA(cudaMalloc(&h->buf, sizeof(float2) * size_t(h->nf) * V));
		MESH_CUDA(cudaMalloc(&h->buf_old, sizeof(float2) * size_t(h->nf) * V));
		MESH_CUDA(cudaMalloc(&h->g_trial, sizeof(double) * size_t(group_nr(U.group)) * V));
		MESH_CUDA(cudaMalloc(&h->red, sizeof(double) * 2 * kMaxRedBlocks));
		MESH_CUDA(cudaMalloc(&h->res, sizeof(double) * 2));
		MESH_CUDA(cudaMalloc(&h->cnt, sizeof(unsigned) * 2));
		MESH_CUDA(cudaMemset(h->cnt, 0, sizeof(unsigned) * 2));
		MomTables &mt = h->mt;
		mt.nd = U.nd;
		int64_t st = 1;
		for (int d = U.nd - 1; d >= 0; --d)
		{
			mt.L[d] = U.dims[d];
			mt.stride[d] = st;
			st *= U.dims[d];
			for (int n = 0; n < 32; ++n)
			{
				double t = std::sin(M_PI * double(n) / double(U.dims[d]));
				mt.s[d][n] = float(4.0 * t * t);
			}
		}
		for (int d = U.nd; d < 4; ++d)
		{
			mt.L[d] = 1;
			mt.stride[d] = 1;
		}
		mt.p2max = 0.f;
		for (int d = 0; d < U.nd; ++d)
		{
			float mx = 0.f;
			for (int n = 0; n < U.dims[d]; ++n)
				mx = std::max(mx, mt.s[d][n]);
			mt.p2max += mx;
		}
		h->mult.mode = 0;
		h->mult.alpha = 0.08f;
	});
	if (rc != MESH_OK)
	{
		delete h;
		return rc;
	}
	*out = h;
	return MESH_OK;
}

int mesh_landau_fa_destroy(mesh_landau_fa_s *h)
{
	if (h)
	{
		if (h->ctx)
			cudaStreamSynchronize(h->ctx->stream);
		delete h;
	}
	return MESH_OK;
}

int mesh_landau_fa_set_plain(mesh_landau_fa_s *h, double alpha)
{
	return fa_api([&] {
		require(h != nullptr && alpha > 0, "invalid argument");
		h->mult.mode = 0;
		h->mult.alpha = float(alpha);
		h->learned = false;
	});
}

// learned multiplier: log m sampled on n points uniform in log p^2 over
// [log_p2_lo, log_p2_hi] (the caller evaluates the network on that grid)
int mesh_landau_fa_set_table(mesh_landau_fa_s *h, float const *log_mult, int n, double log_p2_lo, double log_p2_hi)
{
	return fa_api([&] {
		require(h != nullptr && log_mult != nullptr && n >= 2 && log_p2_hi > log_p2_lo, "invalid argument");
		DeviceGuard dg(h->ctx->device);
		if (int(h->host_table.size()) != n)
		{
			cudaFree(h->table);
			h->table = nullptr;
			MESH_CUDA(cudaMalloc(&h->table, sizeof(float) * size_t(n)));
		}
		h->host_table.assign(log_mult, log_mult + n);
		MESH_CUDA(cudaMemcpyAsync(h->table, log_mult, sizeof(float) * size_t(n), cudaMemcpyHostToDevice,
		                          h->ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
		h->mult.mode = 1;
		h->mult.table = h->table;
		h->mult.n = n;
		h->mult.lo = float(log_p2_lo);
		h->mult.hi = float(log_p2_hi);
		h->learned = false;
	});
}

// learned multiplier: log m = MLP(log p^2 - log p2max, 5 (beta - 6),
// (log10 theta + 7)/5), re-evaluated (BF16 inference when bf16 != 0) on a
// grid of 256 points in log p^2 before every step
int mesh_landau_fa_set_mlp(mesh_landau_fa_s *h, float const *params, int width, double beta, int bf16)
{
	return fa_api([&] {
		require(h != nullptr && params != nullptr && (width == 32 || width == 64), "invalid argument");
		DeviceGuard dg(h->ctx->device);
		int np = 3 * width + width + width * width + width + width + 1;
		cudaFree(h->mlp_params);
		h->mlp_params = nullptr;
		MESH_CUDA(cudaMalloc(&h->mlp_params, sizeof(float) * size_t(np)));
		MESH_CUDA(cudaMemcpyAsync(h->mlp_params, params, sizeof(float) * size_t(np), cudaMemcpyHostToDevice,
		                          h->ctx->stream));
		if (!h->mlp_x)
			MESH_CUDA(cudaMalloc(&h->mlp_x, sizeof(float) * 3 * size_t(h->mlp_n)));
		if (int(h->host_table.size()) != h->mlp_n)
		{
			cudaFree(h->table);
			h->table = nullptr;
			MESH_CUDA(cudaMalloc(&h->table, sizeof(float) * size_t(h->mlp_n)));
			h->host_table.assign(size_t(h->mlp_n), 0.f);
		}
		double p2min = 1e30;
		for (int d = 0; d < h->mt.nd; ++d)
			p2min = std::min(p2min, double(h->mt.s[d][1]));
		h->mlp_width = width;
		h->mlp_bf16 = bf16 != 0;
		h->mlp_beta = beta;
		h->learned = true;
		h->mult.mode = 1;
		h->mult.table = h->table;
		h->mult.n = h->mlp_n;
		h->mult.lo = float(std::log(p2min) - 1e-3);
		h->mult.hi = float(std::log(double(h->mt.p2max)) + 1e-3);
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
	});
}

int mesh_landau_fa_p2range(mesh_landau_fa_s *h, double *p2min, double *p2max)
{
	return fa_api([&] {
		require(h != nullptr, "null workspace");
		float mn = 1e30f;
		for (int d = 0; d < h->mt.nd; ++d)
			if (h->mt.L[d] > 1)
				mn = std::min(mn, h->mt.s[d][1]);
		if (p2min)
			*p2min = mn;
		if (p2max)
			*p2max = h->mt.p2max;
	});
}

// theta_ref of g (FP64), via the same kernels as the step
int mesh_landau_fa_theta(mesh_landau_fa_s *h, mesh_field gh, double *theta)
{
	return fa_api([&] {
		require(h != nullptr && gh != nullptr && theta != nullptr, "null argument");
		Field const &g = gh->f;
		require(g.same_grid(*h->U) && g.group == h->U->group && g.prec == MESH_F64 && g.nstack == 1,
		        "g must be an FP64 site field on U's grid", MESH_ERR_STATE);
		DeviceGuard dg(h->ctx->device);
		*theta = h->theta(g, false);
	});
}

// one step in place; theta_before = theta of g before the step
int mesh_landau_fa_step(mesh_landau_fa_s *h, mesh_field gh, double *theta_before)
{
	return fa_api([&] {
		require(h != nullptr && gh != nullptr, "null argument");
		Field &g = gh->f;
		require(g.same_grid(*h->U) && g.group == h->U->group && g.prec == MESH_F64 && g.nstack == 1,
		        "g must be an FP64 site field on U's grid", MESH_ERR_STATE);
		DeviceGuard dg(h->ctx->device);
		double th = h->theta(g, true);
		if (!std::isfinite(th))
			throw Error(MESH_ERR_NUMERIC, "non-finite gauge condition theta");
		h->step_from_buf(g, static_cast<double *>(g.d), h->mult, th);
		if (theta_before)
			*theta_before = th;
	});
}

int mesh_landau_fa_set_accept(mesh_landau_fa_s *h, int on_functional)
{
	return fa_api([&] {
		require(h != nullptr && (on_functional == 0 || on_functional == 1), "invalid argument");
		h->accept_functional = on_functional == 1;
	});
}

// Steps until theta < tol. Every step is checked: by default a step that did
// not lower theta, with mesh_landau_fa_set_accept(h, 1) one that lowered the
// gauge functional (by more than its FP64 summation error), is undone and
// `or_sweeps` overrelaxation sweeps (omega) run instead. iters counts steps
// taken, fallbacks the OR blocks.
int mesh_landau_fa_run(mesh_landau_fa_s *h, mesh_field gh, double tol, int max_iter, double omega, int or_sweeps,
                       int *iters, int *fallbacks, double *theta_out)
{
	return fa_api([&] {
		require(h != nullptr && gh != nullptr, "null argument");
		Field &g = gh->f;
		require(g.same_grid(*h->U) && g.group == h->U->group && g.prec == MESH_F64 && g.nstack == 1,
		        "g must be an FP64 site field on U's grid", MESH_ERR_STATE);
		require(max_iter >= 0 && or_sweeps >= 1 && omega > 0 && omega < 2, "invalid argument");
		DeviceGuard dg(h->ctx->device);
		auto const &ops = ops_for(*h->U);
		Context &c = *h->ctx;
		Field trial = g;
		trial.d = h->g_trial;
		bool by_f = h->accept_functional;
		double f = 0, f_new = 0;
		double th = h->theta(g, true, by_f ? &f : nullptr);
		// FP64 summation error of the functional sum (Nd V terms of size <= Nc)
		double f_tol = 1e-15 * double(group_nc(h->U->group)) * double(h->U->nd) * double(h->U->geom.V);
		int it = 0, fb = 0;
		while (!(th < tol) && it < max_iter)
		{
			if (!std::isfinite(th))
				throw Error(MESH_ERR_NUMERIC, "non-finite gauge condition theta");
			h->step_from_buf(g, h->g_trial, h->mult, th);
			++it;
			double th_new = h->theta(trial, true, by_f ? &f_new : nullptr);
			if (by_f ? (std::isfinite(th_new) && f_new > f - f_tol) : th_new < th)
			{
				MESH_CUDA(cudaMemcpyAsync(g.d, h->g_trial, g.bytes, cudaMemcpyDeviceToDevice, c.stream));
				th = th_new;
				f = f_new;
			}
			else
			{
				// fallback: overrelaxation on the previous g
				++fb;
				for (int k = 0; k < or_sweeps; ++k)
				{
					ops.landau_or_half(*h->U, g, omega, 0);
					ops.landau_or_half(*h->U, g, omega, 1);
				}
				ops.reunit_exact(g);
				th = h->theta(g, true, by_f ? &f : nullptr);
			}
		}
		if (iters)
			*iters = it;
		if (fallbacks)
			*fallbacks = fb;
		if (theta_out)
			*theta_out = th;
		if (!(th < tol))
			throw Error(MESH_ERR_NOCONV, "Fourier-accelerated gauge fixing did not reach the threshold");
	});
}

// Trial step that leaves g unchanged: the current multiplier, or the plain
// one with `alpha` when alpha > 0; returns theta before and after the step.
int mesh_landau_fa_trial(mesh_landau_fa_s *h, mesh_field gh, double alpha, double *theta_before, double *theta_after)
{
	return fa_api([&] {
		require(h != nullptr && gh != nullptr, "null argument");
		Field &g = gh->f;
		require(g.same_grid(*h->U) && g.group == h->U->group && g.prec == MESH_F64 && g.nstack == 1,
		        "g must be an FP64 site field on U's grid", MESH_ERR_STATE);
		DeviceGuard dg(h->ctx->device);
		double th = h->theta(g, true);
		Multiplier m = h->mult;
		if (alpha > 0)
		{
			m.mode = 0;
			m.alpha = float(alpha);
		}
		h->step_from_buf(g, h->g_trial, m, th);
		Field trial = g;
		trial.d = h->g_trial;
		double th2 = h->theta(trial, false);
		if (theta_before)
			*theta_before = th;
		if (theta_after)
			*theta_after = th2;
	});
}

// Response probe: Delta(g) -> F_old; trial step with the plain multiplier
// scaled by `probe_alpha`; Delta(trial) -> F_new; per log-p^2 bin
// lambda_b = sum (|F_old|^2 - Re<F_new,F_old>)/m0 / sum |F_old|^2.
// Outputs per bin: mean p^2, lambda, weight (sum |F_old|^2), count.
int mesh_landau_fa_probe(mesh_landau_fa_s *h, mesh_field gh, double probe_alpha, int nbins, double *p2_mean,
                         double *lambda, double *weight, double *count, double *theta)
{
	return fa_api([&] {
		require(h != nullptr && gh != nullptr && nbins >= 1 && nbins <= 1024, "invalid argument");
		Field &g = gh->f;
		require(g.same_grid(*h->U) && g.group == h->U->group && g.prec == MESH_F64 && g.nstack == 1,
		        "g must be an FP64 site field on U's grid", MESH_ERR_STATE);
		DeviceGuard dg(h->ctx->device);
		Context &c = *h->ctx;
		int64_t V = h->U->geom.V;
		double th = h->theta(g, true);
		fft::fft_nd<-1>(h->buf, h->U->nd, h->U->dims, h->nf, c.num_sms, c.stream);
		MESH_CUDA(cudaMemcpyAsync(h->buf_old, h->buf, sizeof(float2) * size_t(h->nf) * V, cudaMemcpyDeviceToDevice,
		                          c.stream));
		Multiplier m0{};
		m0.mode = 0;
		m0.alpha = float(probe_alpha);
		k_fa_scale<<<grid_for(c, V, 256), 256, 0, c.stream>>>(h->buf, V, h->nf, h->mt, m0);
		MESH_LAUNCH_CHECK();
		fft::fft_nd<+1>(h->buf, h->U->nd, h->U->dims, h->nf, c.num_sms, c.stream);
		h->tab->update(*h->U, h->buf, g, h->g_trial);
		Field trial = g;
		trial.d = h->g_trial;
		h->tab->links(*h->U, trial, h->A, RedSlot{nullptr, nullptr, nullptr});
		h->tab->div(*h->U, h->A, h->buf, h->slot());
		fft::fft_nd<-1>(h->buf, h->U->nd, h->U->dims, h->nf, c.num_sms, c.stream);
		if (h->shell_bins != nbins)
		{
			cudaFree(h->shell);
			h->shell = nullptr;
			MESH_CUDA(cudaMalloc(&h->shell, sizeof(double) * 4 * size_t(nbins)));
			h->shell_bins = nbins;
		}
		MESH_CUDA(cudaMemsetAsync(h->shell, 0, sizeof(double) * 4 * size_t(nbins), c.stream));
		double p2min = 1e30;
		for (int d = 0; d < h->mt.nd; ++d)
			p2min = std::min(p2min, double(h->mt.s[d][1]));
		float blo = float(std::log(p2min) - 1e-3), bhi = float(std::log(double(h->mt.p2max)) + 1e-3);
		k_fa_shell<<<grid_for(c, V, 256, 2), 256, sizeof(double) * 4 * size_t(nbins), c.stream>>>(
		    h->buf_old, h->buf, V, h->nf, h->mt, m0, nbins, blo, bhi, h->shell, h->shell + nbins,
		    h->shell + 2 * nbins, h->shell + 3 * nbins);
		MESH_LAUNCH_CHECK();
		std::vector<double> hs(4 * size_t(nbins));
		MESH_CUDA(cudaMemcpyAsync(hs.data(), h->shell, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaStreamSynchronize(c.stream));
		for (int b = 0; b < nbins; ++b)
		{
			double num = hs[size_t(b)], den = hs[size_t(nbins + b)], p2 = hs[size_t(2 * nbins + b)],
			       n = hs[size_t(3 * nbins + b)];
			if (p2_mean)
				p2_mean[b] = n > 0 ? p2 / n : std::exp(blo + (bhi - blo) * (b + 0.5) / nbins);
			if (lambda)
				lambda[b] = den > 0 ? num / den : 0.0;
			if (weight)
				weight[b] = den;
			if (count)
				count[b] = n;
		}
		if (theta)
			*theta = th;
	});
}

} // extern "C"

// fft_all of the reference (src/lattice/fft.h:55-58, FFTW on the host): an
// unnormalised FFT over every axis of nf complex fields (host array
// [nf][V] of interleaved FP32 complex, lexicographic sites), on the device
extern "C" int mesh_lattice_fft(mesh_ctx ctx, int nd, int32_t const *dims, int nf, float *data, int sign)
{
	return fa_api([&] {
		require(ctx != nullptr && dims != nullptr && data != nullptr && nf >= 1 && (sign == 1 || sign == -1),
		        "invalid argument");
		require(nd >= 1 && nd <= 4, "1 to 4 dimensions");
		int64_t V = 1;
		for (int i = 0; i < nd; ++i)
		{
			require(fft::supported_extent(dims[i]), "FFT extents must be one of 2,4,6,8,12,16,24,32");
			V *= dims[i];
		}
		Context &c = ctx->c;
		DeviceGuard dg(c.device);
		size_t bytes = sizeof(float2) * size_t(nf) * size_t(V);
		float2 *d = nullptr;
		MESH_CUDA(cudaMallocAsync(&d, bytes, c.stream));
		MESH_CUDA(cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, c.stream));
		if (sign < 0)
			fft::fft_nd<-1>(d, nd, dims, nf, c.num_sms, c.stream);
		else
			fft::fft_nd<+1>(d, nd, dims, nf, c.num_sms, c.stream);
		MESH_LAUNCH_CHECK();
		MESH_CUDA(cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaFreeAsync(d, c.stream));
		MESH_CUDA(cudaStreamSynchronize(c.stream));
	});
}
