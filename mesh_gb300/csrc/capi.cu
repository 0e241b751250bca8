// extern "C" entry points of libmesh_gb300.so: argument checking, layout
// conversion staging, host-side control flow (the HMC trajectory sequence,
// the Landau solvers) over the kernels of kernels.cuh. No exception crosses
// the ABI; every function returns a MESH_* status.
#include "field.cuh"

#include <cmath>
#include <cstring>
#include <exception>
#include <limits>
#include <string>
#include <vector>

using namespace meshgb;

// the context's device error word (bounded device-side waits): reads it
// (synchronising the stream), clears it and reports a nonzero code
void meshgb::check_device_error(Context &c)
{
	int e = 0;
	MESH_CUDA(cudaMemcpyAsync(&e, c.d_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
	MESH_CUDA(cudaStreamSynchronize(c.stream));
	if (e)
	{
		MESH_CUDA(cudaMemsetAsync(c.d_err, 0, sizeof(int), c.stream));
		throw Error(MESH_ERR_TIMEOUT, "a bounded device-side wait expired (a copy or flag it waited for did not "
		                              "arrive); the launch's results are invalid");
	}
}

namespace {
void teardown_ctx(Context &c)
{
	cudaSetDevice(c.device);
	if (c.stream)
		cudaStreamSynchronize(c.stream);
	cudaFree(c.d_partials);
	cudaFree(c.d_results);
	cudaFree(c.d_counters);
	cudaFree(c.d_err);
	if (c.d_stage)
		cudaFree(c.d_stage);
	if (c.own_stream && c.stream)
		cudaStreamDestroy(c.stream);
}

// drops one owner of the context; frees it with the last one
void release_ctx(Context *c)
{
	if (c && --c->refs == 0)
	{
		teardown_ctx(*c);
		delete reinterpret_cast<mesh_ctx_s *>(c);
	}
}
} // namespace

namespace {
thread_local std::string g_err;
} // namespace

void meshgb::set_last_error(char const *msg) { g_err = msg; }

namespace {
int fail(int code, char const *msg)
{
	g_err = msg;
	return code;
}

template <class F> int api(F &&f) { return api_call(f); }

Field &F(mesh_field h)
{
	require(h != nullptr, "null field handle");
	return h->f;
}

double read_slot(Context &c, int k)
{
	double v = 0;
	MESH_CUDA(cudaMemcpyAsync(&v, c.d_results + k, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
	MESH_CUDA(cudaStreamSynchronize(c.stream));
	return v;
}

void create_field(Context &c, int kind, int group, int prec, int nd, int32_t const *dims, int nstack, Field &f)
{
	require(kind == MESH_GROUP || kind == MESH_ALGEBRA, "kind must be MESH_GROUP or MESH_ALGEBRA");
	require(group >= 1 && group <= 3, "unknown gauge group");
	require(prec == MESH_F32 || prec == MESH_F64, "invalid precision level");
	require(nd >= 2 && nd <= 4, "number of dimensions must be 2, 3 or 4");
	require(dims != nullptr, "null dims");
	require(nstack >= 1 && nstack <= 64, "nstack must be in [1, 64]");
	int64_t V = 1;
	for (int i = 0; i < nd; ++i)
	{
		require(dims[i] >= 2 && dims[i] % 2 == 0, "every extent must be even and >= 2 (checkerboard layout)");
		require(dims[i] < 256, "every extent must be below 256");
		V *= dims[i];
		require(V < (int64_t(1) << 31), "volume must be below 2^31");
	}
	f.ctx = &c;
	f.kind = kind;
	f.group = group;
	f.prec = prec;
	f.nd = nd;
	f.nstack = nstack;
	for (int i = 0; i < 4; ++i)
		f.dims[i] = i < nd ? dims[i] : 0;
	f.geom = make_geom(nd, dims);
	f.nr = kind == MESH_GROUP ? group_nr(group) : group_na(group);
	f.nr_host = group_nr(group);
	f.real_bytes = prec == MESH_F32 ? 4 : 8;
	f.bytes = size_t(nstack) * size_t(V) * size_t(f.nr) * f.real_bytes;
	DeviceGuard dg(c.device);
	MESH_CUDA(cudaMalloc(&f.d, f.bytes));
	++c.refs;
}

void destroy_field(Field &f)
{
	if (f.d)
	{
		{
			DeviceGuard dg(f.ctx->device);
			cudaStreamSynchronize(f.ctx->stream);
			cudaFree(f.d);
		}
		release_ctx(f.ctx);
	}
	f.d = nullptr;
	f.ctx = nullptr;
}

void same_shape(Field const &a, Field const &b)
{
	require(a.same_grid(b) && a.group == b.group && a.prec == b.prec, "fields on different grids/groups/precisions",
	        MESH_ERR_STATE);
}

double nplanes(int nd) { return nd * (nd - 1) * 0.5; }

// the device address of a pinned (page-locked, mapped) host buffer that a
// kernel may read and write directly, 16-byte aligned; nullptr otherwise
// (pageable memory goes through a staging copy)
static void *mapped_host(void const *host)
{
	if (reinterpret_cast<uintptr_t>(host) % 16 != 0)
		return nullptr;
	cudaPointerAttributes a{};
	if (cudaPointerGetAttributes(&a, host) != cudaSuccess)
	{
		cudaGetLastError();
		return nullptr;
	}
	return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// MESH_HOST_PATH=staged: pinned host buffers too go through the staging copy
// (one DMA copy, then the conversion kernel on the device) instead of the
// conversion kernel reading or writing the mapped host memory
static bool force_staged()
{
	char const *e = std::getenv("MESH_HOST_PATH");
	return e && std::strcmp(e, "staged") == 0;
}

void import_host(Field &f, void const *host, size_t bytes)
{
	require(host != nullptr, "null host buffer");
	require(bytes == f.host_bytes(), "host buffer size does not match the field");
	auto &c = *f.ctx;
	DeviceGuard dg(c.device);
	if (void *d = force_staged() ? nullptr : mapped_host(host))
	{
		ops_for(f).import_direct(f, d);
		MESH_CUDA(cudaStreamSynchronize(c.stream));
		return;
	}
	void *stage = c.stage(bytes);
	MESH_CUDA(cudaMemcpyAsync(stage, host, bytes, cudaMemcpyHostToDevice, c.stream));
	ops_for(f).import_(f, stage);
	MESH_CUDA(cudaStreamSynchronize(c.stream));
}

void export_host(Field const &f, void *host, size_t bytes)
{
	require(host != nullptr, "null host buffer");
	require(bytes == f.host_bytes(), "host buffer size does not match the field");
	auto &c = *f.ctx;
	DeviceGuard dg(c.device);
	if (void *d = force_staged() ? nullptr : mapped_host(host))
	{
		ops_for(f).export_direct(f, d);
		MESH_CUDA(cudaStreamSynchronize(c.stream));
		return;
	}
	void *stage = c.stage(bytes);
	ops_for(f).export_(f, stage);
	MESH_CUDA(cudaMemcpyAsync(host, stage, bytes, cudaMemcpyDeviceToHost, c.stream));
	MESH_CUDA(cudaStreamSynchronize(c.stream));
}

// makeDeltas (src/gauge/hmc.cpp:7-51): base pattern per scheme, substeps
// joined by merging the touching end steps, scaled by sqrt(2 eps)/substeps
std::vector<double> make_deltas(std::string const &scheme, double epsilon, int substeps)
{
	require(substeps >= 1, "substeps must be >= 1");
	require(epsilon > 0, "epsilon must be > 0");
	double delta = std::sqrt(2 * epsilon) / substeps;
	std::vector<double> raw;
	if (scheme == "2lf")
		raw = {0.5, 1.0, 0.5};
	else if (scheme == "2mn")
	{
		double lamb = 0.19318332750378361;
		raw = {lamb, 0.5, 1.0 - 2.0 * lamb, 0.5, lamb};
	}
	else if (scheme == "4mn")
	{
		double rho = 0.1786178958448091;
		double theta = -0.06626458266981843;
		double lamb = 0.7123418310626056;
		raw = {rho, lamb, theta, 0.5 - lamb, 1.0 - 2.0 * (rho + theta), 0.5 - lamb, theta, lamb, rho};
	}
	else
		throw Error(MESH_ERR_ARG, "unknown scheme '" + scheme + "'");
	std::vector<double> d;
	d.reserve((raw.size() - 1) * size_t(substeps) + 1);
	for (int i = 0; i < substeps; ++i)
	{
		if (i == 0)
			d.insert(d.end(), raw.begin(), raw.end());
		else
		{
			d.back() *= 2;
			d.insert(d.end(), raw.begin() + 1, raw.end());
		}
	}
	for (double &x : d)
		x *= delta;
	return d;
}

void check_deltas(double const *deltas, int n)
{
	require(deltas != nullptr && n >= 1, "empty step table");
	require(n % 2 == 1, "step table must alternate position/momentum steps and have odd length");
}

// out = a x + b y over every stored real, y optional; out may be x or y (no
// restrict). One thread per real in a grid-stride loop: consecutive threads
// read consecutive words of each array.
template <class T>
__global__ void __launch_bounds__(256) k_axpby(int64_t n, T a, T const *x, T b, T const *y, T *out)
{
	for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
		out[i] = y ? a * x[i] + b * y[i] : a * x[i];
}

} // namespace

void meshgb::ctx_retain(Context &c) { ++c.refs; }
void meshgb::ctx_release(Context *c) { release_ctx(c); }
void meshgb::field_import_host(Field &f, void const *host, size_t bytes) { import_host(f, host, bytes); }
void meshgb::field_export_host(Field const &f, void *host, size_t bytes) { export_host(f, host, bytes); }

// ---------------------------------------------------------------------------
// HMC chain state
// ---------------------------------------------------------------------------
struct mesh_hmc_s
{
	Context *ctx = nullptr;
	// U: the chain's configuration; Unew: the proposal; Ut: the second buffer
	// of the fused momentum-step + link-update kernels, which write the links
	// out of place (Unew and Ut alternate)
	mesh_field_s U, Unew, Ut, P;
	uint64_t seed = 0;
	HmcDev *d_dev = nullptr;
	HmcRecordDev *d_hist = nullptr;
	// private FP64 reduction slots (a context may hold several chains)
	double *d_part = nullptr, *d_res = nullptr;
	unsigned *d_cnt = nullptr;
	int hist_cap = 0;
	int *d_flag = nullptr;
	int64_t count = 0; // trajectories enqueued
	bool S_valid = false;
	// cached CUDA graph of one trajectory
	cudaGraphExec_t graph = nullptr;
	double graph_beta = 0;
	std::vector<double> graph_deltas;
	HmcRecordDev *graph_hist = nullptr;

	enum
	{
		S_CUR = 0,
		K_OLD = 1,
		S_NEW = 2,
		K_NEW = 3,
		NSLOT = 4
	};
	RedSlot rs(int k) { return {d_part + size_t(k) * kMaxRedBlocks, d_res + k, d_cnt + k}; }

	void drop_graph()
	{
		if (graph)
			cudaGraphExecDestroy(graph);
		graph = nullptr;
	}

	void ensure_history(int64_t need)
	{
		if (need <= hist_cap)
			return;
		int cap = hist_cap ? hist_cap : 1024;
		while (cap < need)
			cap *= 2;
		HmcRecordDev *nh = nullptr;
		MESH_CUDA(cudaMallocAsync(&nh, size_t(cap) * sizeof(HmcRecordDev), ctx->stream));
		if (d_hist)
		{
			MESH_CUDA(cudaMemcpyAsync(nh, d_hist, size_t(hist_cap) * sizeof(HmcRecordDev), cudaMemcpyDeviceToDevice,
			                          ctx->stream));
			MESH_CUDA(cudaFreeAsync(d_hist, ctx->stream));
		}
		d_hist = nh;
		hist_cap = cap;
		MESH_CUDA(cudaMemcpyAsync(&d_dev->history_cap, &hist_cap, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		drop_graph();
	}

	// Enqueue one trajectory (runHmcUpdate, hmc.cpp:73-107) on the stream.
	// P0 != nullptr: supplied momenta; uniform NaN: draw from the stream.
	void enqueue(double beta, double const *deltas, int n, Field const *P0, double uniform)
	{
		Field &u = U.f, &un = Unew.f, &p = P.f;
		auto const &ops = ops_for(u);
		Context &c = *ctx;
		if (!S_valid)
		{
			ops.hmc_plaquette(u, rs(S_CUR));
			S_valid = true;
		}
		if (P0)
		{
			MESH_CUDA(cudaMemcpyAsync(p.d, P0->d, p.bytes, cudaMemcpyDeviceToDevice, c.stream));
			ops.norm2(p, rs(K_OLD));
		}
		else
			ops.random_momenta_dev(p, seed, &d_dev->traj, rs(K_OLD));
		double coef0 = beta / (2.0 * group_nc(u.group));
		int last_p = n >= 3 ? n - 2 : -1;
		// the proposal: built in Unew (and Ut, when momentum steps are fused
		// with the link updates after them)
		Field *cur = &un, *spare = &Ut.f;
		for (int i = 0; i < n; ++i)
		{
			if (i % 2 == 0)
				ops.hmc_evolve(i == 0 ? u : *cur, *cur, p, deltas[i], i == n - 1);
			else
			{
				RedSlot kin = rs(K_NEW);
				RedSlot *k = i == last_p ? &kin : nullptr;
				if (i + 1 < n && ops.hmc_md_step(p, *cur, *spare, coef0 * deltas[i], deltas[i + 1], i + 1 == n - 1, k))
				{
					std::swap(cur, spare);
					++i; // the link update i + 1 is done
				}
				else
					ops.hmc_momentum_step(p, *cur, coef0 * deltas[i], k);
			}
		}
		if (last_p < 0)
			ops.norm2(p, rs(K_NEW));
		ops.hmc_plaquette(*cur, rs(S_NEW));
		double *res = d_res;
		launch_metropolis(c, d_dev, d_hist, res + S_CUR, res + K_OLD, res + S_NEW, res + K_NEW, res + S_CUR, beta,
		                  nplanes(u.nd) * double(u.geom.V), double(group_nc(u.group)), seed, uniform, d_flag);
		launch_copy_if(c, u.d, cur->d, u.bytes, d_flag);
		++count;
	}

	HmcRecordDev record(int64_t k)
	{
		HmcRecordDev r;
		MESH_CUDA(cudaMemcpyAsync(&r, d_hist + k, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		return r;
	}

	void check_bad()
	{
		check_device_error(*ctx);
		int bad = 0;
		MESH_CUDA(cudaMemcpyAsync(&bad, &d_dev->bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		if (bad)
		{
			int zero = 0;
			cudaMemcpy(&d_dev->bad, &zero, sizeof(int), cudaMemcpyHostToDevice);
			throw Error(MESH_ERR_NUMERIC, "non-finite Hamiltonian in HMC trajectory (trajectory rejected)");
		}
	}
};

extern "C" {

char const *mesh_last_error(void) { return g_err.c_str(); }
int mesh_version(void) { return 100; }

// ---- context ---------------------------------------------------------------
int mesh_ctx_create(int device, void *stream, mesh_ctx *out)
{
	if (!out)
		return fail(MESH_ERR_ARG, "null output handle");
	*out = nullptr;
	auto *h = new mesh_ctx_s();
	int rc = api([&] {
		Context &c = h->c;
		int n = 0;
		MESH_CUDA(cudaGetDeviceCount(&n));
		require(device >= 0 && device < n, "device index out of range");
		c.device = device;
		DeviceGuard dg(device);
		MESH_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
		if (stream)
			c.stream = static_cast<cudaStream_t>(stream);
		else
		{
			MESH_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
			c.own_stream = true;
		}
		MESH_CUDA(cudaMalloc(&c.d_partials, sizeof(double) * size_t(kSlots) * kMaxRedBlocks));
		MESH_CUDA(cudaMalloc(&c.d_results, sizeof(double) * kSlots));
		MESH_CUDA(cudaMalloc(&c.d_counters, sizeof(unsigned) * kSlots));
		MESH_CUDA(cudaMemset(c.d_counters, 0, sizeof(unsigned) * kSlots));
		MESH_CUDA(cudaMemset(c.d_results, 0, sizeof(double) * kSlots));
		MESH_CUDA(cudaMalloc(&c.d_err, sizeof(int)));
		MESH_CUDA(cudaMemset(c.d_err, 0, sizeof(int)));
	});
	if (rc != MESH_OK)
	{
		mesh_ctx_destroy(h);
		return rc;
	}
	*out = h;
	return MESH_OK;
}

int mesh_ctx_destroy(mesh_ctx h)
{
	// releases the caller's reference; fields and chains still alive keep
	// the context until they are destroyed
	if (h)
		release_ctx(&h->c);
	return MESH_OK;
}

int mesh_ctx_synchronize(mesh_ctx h)
{
	return api([&] {
		require(h != nullptr, "null context");
		MESH_CUDA(cudaStreamSynchronize(h->c.stream));
		check_device_error(h->c);
	});
}

void *mesh_ctx_stream(mesh_ctx h) { return h ? static_cast<void *>(h->c.stream) : nullptr; }

namespace {
// one thread waits for *flag != 0, giving up after limit_ns (global timer)
// and recording that in the context's device error word, as the kernels
// with bounded waits do
__global__ void k_wait_probe(unsigned const *flag, int *err, unsigned long long limit_ns)
{
	auto now = [] {
		unsigned long long t;
		asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
		return t;
	};
	unsigned long long t0 = now();
	while (atomicAdd(const_cast<unsigned *>(flag), 0u) == 0u)
	{
		if (now() - t0 > limit_ns)
		{
			atomicExch(err, 1);
			return;
		}
		__nanosleep(1000);
	}
}
} // namespace

int mesh_ctx_wait_probe(mesh_ctx h, double seconds, int flag_set)
{
	return api([&] {
		require(h != nullptr, "null context");
		require(seconds > 0 && seconds <= 2.0, "wait limit must be in (0, 2] seconds");
		auto &c = h->c;
		DeviceGuard dg(c.device);
		unsigned *flag = nullptr;
		MESH_CUDA(cudaMalloc(&flag, sizeof(unsigned)));
		cudaError_t e = cudaMemsetAsync(flag, flag_set ? 1 : 0, sizeof(unsigned), c.stream);
		if (e == cudaSuccess)
		{
			k_wait_probe<<<1, 1, 0, c.stream>>>(flag, c.d_err, (unsigned long long)(seconds * 1e9));
			e = cudaGetLastError();
		}
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(c.stream);
		cudaFree(flag);
		MESH_CUDA(e);
		check_device_error(c);
	});
}

// ---- fields ----------------------------------------------------------------
int mesh_field_create(mesh_ctx ctx, int kind, int group, int precision, int nd, int32_t const *dims, int nstack,
                      mesh_field *out)
{
	if (!out)
		return fail(MESH_ERR_ARG, "null output handle");
	*out = nullptr;
	if (!ctx)
		return fail(MESH_ERR_ARG, "null context");
	auto *h = new mesh_field_s();
	int rc = api([&] { create_field(ctx->c, kind, group, precision, nd, dims, nstack, h->f); });
	if (rc != MESH_OK)
	{
		delete h;
		return rc;
	}
	*out = h;
	return MESH_OK;
}

int mesh_field_destroy(mesh_field h)
{
	if (!h)
		return MESH_OK;
	destroy_field(h->f);
	delete h;
	return MESH_OK;
}

int mesh_field_info(mesh_field h, int *kind, int *group, int *precision, int *nd, int32_t *dims, int *nstack)
{
	return api([&] {
		Field &f = F(h);
		if (kind)
			*kind = f.kind;
		if (group)
			*group = f.group;
		if (precision)
			*precision = f.prec;
		if (nd)
			*nd = f.nd;
		if (dims)
			for (int i = 0; i < f.nd; ++i)
				dims[i] = f.dims[i];
		if (nstack)
			*nstack = f.nstack;
	});
}

size_t mesh_field_host_bytes(mesh_field h) { return h ? h->f.host_bytes() : 0; }

int mesh_field_import(mesh_field h, void const *host, size_t bytes)
{
	return api([&] { import_host(F(h), host, bytes); });
}

int mesh_field_export(mesh_field h, void *host, size_t bytes)
{
	return api([&] { export_host(F(h), host, bytes); });
}

// ---- configuration files ---------------------------------------------------
int mesh_field_save(mesh_field h, char const *path)
{
	return api([&] {
		Field const &f = F(h);
		std::vector<unsigned char> buf(f.host_bytes());
		export_host(f, buf.data(), buf.size());
		config_write(path, config_header_of(f, 0, 0), buf.data(), buf.size());
	});
}

int mesh_field_load(mesh_field h, char const *path)
{
	return api([&] {
		Field &f = F(h);
		ConfigHeader hd = config_read_header(path);
		config_check_matches(hd, f);
		std::vector<unsigned char> buf(f.host_bytes());
		config_read_data(path, hd, buf.data(), buf.size());
		import_host(f, buf.data(), buf.size());
	});
}

int mesh_config_info(char const *path, int *kind, int *group, int *precision, int *nd, int32_t *dims, int *nstack,
                     uint64_t *trajectory, uint64_t *seed)
{
	return api([&] {
		ConfigHeader hd = config_read_header(path);
		if (kind)
			*kind = hd.kind;
		if (group)
			*group = hd.group;
		if (precision)
			*precision = hd.precision;
		if (nd)
			*nd = hd.nd;
		if (dims)
			for (int i = 0; i < hd.nd; ++i)
				dims[i] = hd.dims[i];
		if (nstack)
			*nstack = hd.nstack;
		if (trajectory)
			*trajectory = hd.trajectory;
		if (seed)
			*seed = hd.seed;
	});
}

int mesh_field_copy(mesh_field dst, mesh_field src)
{
	return api([&] {
		Field &d = F(dst), &s = F(src);
		same_shape(d, s);
		require(d.kind == s.kind && d.nstack == s.nstack, "fields differ in kind or stack size", MESH_ERR_STATE);
		DeviceGuard dg(d.ctx->device);
		MESH_CUDA(cudaMemcpyAsync(d.d, s.d, d.bytes, cudaMemcpyDeviceToDevice, d.ctx->stream));
	});
}

int mesh_field_set_zero(mesh_field h)
{
	return api([&] {
		Field &f = F(h);
		DeviceGuard dg(f.ctx->device);
		MESH_CUDA(cudaMemsetAsync(f.d, 0, f.bytes, f.ctx->stream));
	});
}

int mesh_field_set_unit(mesh_field h)
{
	return api([&] {
		Field &f = F(h);
		require(f.kind == MESH_GROUP, "set_unit needs a group field");
		DeviceGuard dg(f.ctx->device);
		ops_for(f).set_unit(f);
	});
}

int mesh_field_random(mesh_field h, uint64_t seed, uint64_t counter)
{
	return api([&] {
		Field &f = F(h);
		DeviceGuard dg(f.ctx->device);
		ops_for(f).random(f, seed, counter, RedSlot{});
	});
}

void *mesh_field_device_ptr(mesh_field h) { return h ? h->f.d : nullptr; }

// ---- lattice layer ---------------------------------------------------------
int mesh_site_cshift(mesh_field dst, mesh_field src, int dir, int offset)
{
	return api([&] {
		Field &d = F(dst), &s = F(src);
		same_shape(d, s);
		require(d.kind == MESH_GROUP && s.kind == MESH_GROUP && d.nstack == 1 && s.nstack == 1,
		        "cshift operates on single-component group fields");
		require(dir >= 0 && dir < d.nd, "direction out of range");
		require(d.d != s.d, "inplace cshift not supported");
		DeviceGuard dg(d.ctx->device);
		ops_for(d).cshift(d, s, dir, offset);
	});
}

int mesh_site_mul(mesh_field dst, mesh_field a, mesh_field b)
{
	return api([&] {
		Field &d = F(dst), &x = F(a), &y = F(b);
		same_shape(d, x);
		same_shape(d, y);
		require(d.kind == MESH_GROUP && x.kind == MESH_GROUP && y.kind == MESH_GROUP && d.nstack == 1 &&
		            x.nstack == 1 && y.nstack == 1,
		        "site_mul operates on single-component group fields");
		DeviceGuard dg(d.ctx->device);
		ops_for(d).site_op(SITE_MUL, d, x, &y);
	});
}

int mesh_field_axpby(mesh_field out, double a, mesh_field x, double b, mesh_field y)
{
	return api([&] {
		require(out != nullptr && x != nullptr, "null field");
		Field &o = F(out), &u = F(x);
		same_shape(o, u);
		require(o.kind == u.kind && o.nstack == u.nstack, "fields differ in kind or stack size", MESH_ERR_STATE);
		Field *v = y ? &F(y) : nullptr;
		if (v)
		{
			same_shape(o, *v);
			require(o.kind == v->kind && o.nstack == v->nstack, "fields differ in kind or stack size", MESH_ERR_STATE);
		}
		int64_t n = int64_t(o.bytes / o.real_bytes);
		Context &c = *o.ctx;
		DeviceGuard dg(c.device);
		unsigned blocks = grid_for(c, n, 256);
		if (o.prec == MESH_F32)
			k_axpby<float><<<blocks, 256, 0, c.stream>>>(n, float(a), static_cast<float const *>(u.d), float(b),
			                                             v ? static_cast<float const *>(v->d) : nullptr,
			                                             static_cast<float *>(o.d));
		else
			k_axpby<double><<<blocks, 256, 0, c.stream>>>(n, a, static_cast<double const *>(u.d), b,
			                                              v ? static_cast<double const *>(v->d) : nullptr,
			                                              static_cast<double *>(o.d));
		MESH_LAUNCH_CHECK();
	});
}

int mesh_site_exp(mesh_field dst, mesh_field a)
{
	return api([&] {
		Field &d = F(dst), &x = F(a);
		same_shape(d, x);
		require(d.kind == MESH_GROUP && x.kind == MESH_ALGEBRA && d.nstack == 1 && x.nstack == 1,
		        "site_exp maps a single-component algebra field to a group field");
		DeviceGuard dg(d.ctx->device);
		ops_for(d).site_op(SITE_EXP, d, x, nullptr);
	});
}

int mesh_site_project(mesh_field dst, mesh_field a)
{
	return api([&] {
		Field &d = F(dst), &x = F(a);
		same_shape(d, x);
		require(d.kind == MESH_ALGEBRA && x.kind == MESH_GROUP && d.nstack == 1 && x.nstack == 1,
		        "site_project maps a single-component group field to an algebra field");
		DeviceGuard dg(d.ctx->device);
		ops_for(d).site_op(SITE_PROJ, d, x, nullptr);
	});
}

int mesh_site_adj(mesh_field dst, mesh_field a)
{
	return api([&] {
		Field &d = F(dst), &x = F(a);
		same_shape(d, x);
		require(d.kind == MESH_GROUP && x.kind == MESH_GROUP && d.nstack == 1 && x.nstack == 1,
		        "site_adj operates on single-component group fields");
		DeviceGuard dg(d.ctx->device);
		ops_for(d).site_op(SITE_ADJ, d, x, nullptr);
	});
}

int mesh_site_sum_real_trace(mesh_field a, double *out)
{
	return api([&] {
		Field &x = F(a);
		require(out != nullptr, "null output");
		require(x.kind == MESH_GROUP && x.nstack == 1, "sum_real_trace operates on a single-component group field");
		DeviceGuard dg(x.ctx->device);
		ops_for(x).sum_real_trace(x, slot(*x.ctx, SLOT_TMP));
		*out = read_slot(*x.ctx, SLOT_TMP);
	});
}

int mesh_field_norm2(mesh_field a, double *out)
{
	return api([&] {
		Field &x = F(a);
		require(out != nullptr, "null output");
		DeviceGuard dg(x.ctx->device);
		ops_for(x).norm2(x, slot(*x.ctx, SLOT_TMP));
		*out = read_slot(*x.ctx, SLOT_TMP);
	});
}

// ---- gauge -----------------------------------------------------------------
static void check_gauge(Field const &U)
{
	require(U.kind == MESH_GROUP && U.nstack == U.nd, "expected a gauge field (group kind, nstack == nd)");
}

int mesh_plaquette(mesh_field Uh, double *out)
{
	return api([&] {
		Field &U = F(Uh);
		check_gauge(U);
		require(out != nullptr, "null output");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).plaquette(U, slot(*U.ctx, SLOT_TMP));
		double s = read_slot(*U.ctx, SLOT_TMP);
		*out = s / (double(U.geom.V) * nplanes(U.nd)) / group_nc(U.group);
	});
}

int mesh_heatbath_sweep(mesh_field Uh, double beta, uint64_t seed, uint64_t sweep)
{
	return api([&] {
		Field &U = F(Uh);
		check_gauge(U);
		require(std::isfinite(beta) && beta >= 0, "beta must be finite and >= 0");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).gauge_sweep(U, beta, seed, sweep, false);
	});
}

int mesh_overrelax_sweep(mesh_field Uh)
{
	return api([&] {
		Field &U = F(Uh);
		check_gauge(U);
		DeviceGuard dg(U.ctx->device);
		ops_for(U).gauge_sweep(U, 0.0, 0, 0, true);
	});
}

int mesh_wilson_loops(mesh_field Uh, int max_r, int max_t, double *out)
{
	return api([&] {
		Field &U = F(Uh);
		check_gauge(U);
		require(out != nullptr, "null output");
		require(U.nd == 4, "Wilson loops need a 4D lattice");
		int lmin = std::min(U.dims[0], std::min(U.dims[1], U.dims[2]));
		require(max_r >= 1 && max_r <= lmin, "max_r must be in 1..min(L0, L1, L2)");
		require(max_t >= 1 && max_t <= U.dims[3], "max_t must be in 1..L3");
		DeviceGuard dg(U.ctx->device);
		Context &c = *U.ctx;
		auto const &ops = ops_for(U);
		size_t comp = size_t(U.geom.V) * size_t(U.nr) * U.real_bytes;
		size_t nres = size_t(max_r) * size_t(max_t);
		char *lines = nullptr; // max_t temporal lines, then the three spatial lines
		double *res = nullptr;
		MESH_CUDA(cudaMallocAsync(&lines, comp * size_t(max_t + 3), c.stream));
		MESH_CUDA(cudaMallocAsync(&res, nres * sizeof(double), c.stream));
		auto release = [&] {
			cudaFreeAsync(lines, c.stream);
			cudaFreeAsync(res, c.stream);
		};
		try
		{
			char *T1 = lines, *S = lines + comp * size_t(max_t);
			char const *u = static_cast<char const *>(U.d);
			MESH_CUDA(cudaMemcpyAsync(T1, u + 3 * comp, comp, cudaMemcpyDeviceToDevice, c.stream));
			for (int t = 2; t <= max_t; ++t)
				ops.line_extend(U, 3, t, T1 + comp * size_t(t - 2), T1 + comp * size_t(t - 1));
			MESH_CUDA(cudaMemcpyAsync(S, u, 3 * comp, cudaMemcpyDeviceToDevice, c.stream));
			RedSlot base = slot(c, SLOT_TMP);
			for (int r = 1; r <= max_r; ++r)
			{
				if (r > 1)
					for (int mu = 0; mu < 3; ++mu)
						ops.line_extend(U, mu, r, S + comp * mu, S + comp * mu);
				for (int t = 1; t <= max_t; ++t)
					ops.wilson_rt(U, r, t, S, T1 + comp * size_t(t - 1),
					              RedSlot{base.partials, res + size_t(r - 1) * max_t + (t - 1), base.counter});
			}
			MESH_CUDA(cudaMemcpyAsync(out, res, nres * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
			MESH_CUDA(cudaStreamSynchronize(c.stream));
		}
		catch (...)
		{
			release();
			throw;
		}
		release();
		double norm = 3.0 * double(U.geom.V) * double(group_nc(U.group));
		for (size_t k = 0; k < nres; ++k)
			out[k] /= norm;
	});
}

int mesh_wilson_action(mesh_field Uh, double beta, double *out)
{
	return api([&] {
		Field &U = F(Uh);
		check_gauge(U);
		require(out != nullptr, "null output");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).plaquette(U, slot(*U.ctx, SLOT_TMP));
		double s = read_slot(*U.ctx, SLOT_TMP);
		double vol = double(U.geom.V);
		double plaq = s / (vol * nplanes(U.nd)) / group_nc(U.group);
		*out = (1.0 - plaq) * (beta * nplanes(U.nd) * vol);
		if (!std::isfinite(*out))
			throw Error(MESH_ERR_NUMERIC, "non-finite Wilson action");
	});
}

int mesh_staple_sum(mesh_field Sh, mesh_field Uh, int mu)
{
	return api([&] {
		Field &S = F(Sh), &U = F(Uh);
		check_gauge(U);
		same_shape(S, U);
		require(S.kind == MESH_GROUP && S.nstack == 1, "staple output must be a single-component group field");
		require(mu >= 0 && mu < U.nd, "direction out of range");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).staple_sum(S, U, mu);
	});
}

int mesh_wilson_deriv(mesh_field Fh, mesh_field Uh, int mu, double beta)
{
	return api([&] {
		Field &Fo = F(Fh), &U = F(Uh);
		check_gauge(U);
		same_shape(Fo, U);
		require(Fo.kind == MESH_ALGEBRA && Fo.nstack == 1, "force output must be a single-component algebra field");
		require(mu >= 0 && mu < U.nd, "direction out of range");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).wilson_deriv(Fo, U, mu, beta);
	});
}

int mesh_reunitize(mesh_field Uh)
{
	return api([&] {
		Field &U = F(Uh);
		require(U.kind == MESH_GROUP, "reunitize needs a group field");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).reunitize(U);
	});
}

int mesh_evolve(mesh_field Uh, mesh_field Ph, double t)
{
	return api([&] {
		Field &U = F(Uh), &P = F(Ph);
		check_gauge(U);
		same_shape(U, P);
		require(P.kind == MESH_ALGEBRA && P.nstack == U.nstack, "momenta must be an algebra field like U");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).evolve(U, U, P, t, false);
	});
}

int mesh_momentum_step(mesh_field Ph, mesh_field Uh, double beta, double delta)
{
	return api([&] {
		Field &U = F(Uh), &P = F(Ph);
		check_gauge(U);
		same_shape(U, P);
		require(P.kind == MESH_ALGEBRA && P.nstack == U.nstack, "momenta must be an algebra field like U");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).momentum_step(P, U, beta / (2.0 * group_nc(U.group)) * delta, nullptr);
	});
}

int mesh_run_hmd(mesh_field Uh, mesh_field Ph, double beta, double const *deltas, int n)
{
	return api([&] {
		Field &U = F(Uh), &P = F(Ph);
		check_gauge(U);
		same_shape(U, P);
		require(P.kind == MESH_ALGEBRA && P.nstack == U.nstack, "momenta must be an algebra field like U");
		check_deltas(deltas, n);
		DeviceGuard dg(U.ctx->device);
		auto const &ops = ops_for(U);
		double coef0 = beta / (2.0 * group_nc(U.group));
		for (int i = 0; i < n; ++i)
			if (i % 2 == 0)
				ops.evolve(U, U, P, deltas[i], false);
			else
				ops.momentum_step(P, U, coef0 * deltas[i], nullptr);
	});
}

int mesh_make_deltas(char const *scheme, double epsilon, int substeps, double *out, int capacity, int *n)
{
	return api([&] {
		require(scheme != nullptr && n != nullptr, "null argument");
		auto d = make_deltas(scheme, epsilon, substeps);
		*n = int(d.size());
		require(out != nullptr && capacity >= int(d.size()), "output buffer too small");
		std::copy(d.begin(), d.end(), out);
	});
}

// ---- HMC -------------------------------------------------------------------
int mesh_hmc_create(mesh_ctx ctx, int group, int precision, int nd, int32_t const *dims, uint64_t seed,
                    mesh_hmc *out)
{
	if (!out)
		return fail(MESH_ERR_ARG, "null output handle");
	*out = nullptr;
	if (!ctx)
		return fail(MESH_ERR_ARG, "null context");
	auto *h = new mesh_hmc_s();
	int rc = api([&] {
		Context &c = ctx->c;
		h->ctx = &c;
		h->seed = seed;
		create_field(c, MESH_GROUP, group, precision, nd, dims, nd, h->U.f);
		create_field(c, MESH_GROUP, group, precision, nd, dims, nd, h->Unew.f);
		create_field(c, MESH_GROUP, group, precision, nd, dims, nd, h->Ut.f);
		create_field(c, MESH_ALGEBRA, group, precision, nd, dims, nd, h->P.f);
		DeviceGuard dg(c.device);
		MESH_CUDA(cudaMalloc(&h->d_dev, sizeof(HmcDev)));
		MESH_CUDA(cudaMemset(h->d_dev, 0, sizeof(HmcDev)));
		MESH_CUDA(cudaMalloc(&h->d_flag, sizeof(int)));
		MESH_CUDA(cudaMemset(h->d_flag, 0, sizeof(int)));
		MESH_CUDA(cudaMalloc(&h->d_part, sizeof(double) * size_t(mesh_hmc_s::NSLOT) * kMaxRedBlocks));
		MESH_CUDA(cudaMalloc(&h->d_res, sizeof(double) * mesh_hmc_s::NSLOT));
		MESH_CUDA(cudaMalloc(&h->d_cnt, sizeof(unsigned) * mesh_hmc_s::NSLOT));
		MESH_CUDA(cudaMemset(h->d_cnt, 0, sizeof(unsigned) * mesh_hmc_s::NSLOT));
		MESH_CUDA(cudaMemset(h->d_res, 0, sizeof(double) * mesh_hmc_s::NSLOT));
		h->ensure_history(1024);
		ops_for(h->U.f).set_unit(h->U.f);
	});
	if (rc != MESH_OK)
	{
		mesh_hmc_destroy(h);
		return rc;
	}
	*out = h;
	return MESH_OK;
}

int mesh_hmc_destroy(mesh_hmc h)
{
	if (!h)
		return MESH_OK;
	if (h->ctx)
	{
		cudaSetDevice(h->ctx->device);
		cudaStreamSynchronize(h->ctx->stream);
		h->drop_graph();
		cudaFree(h->d_dev);
		cudaFree(h->d_hist);
		cudaFree(h->d_flag);
		cudaFree(h->d_part);
		cudaFree(h->d_res);
		cudaFree(h->d_cnt);
		// the fields hold the chain's references to the context
		destroy_field(h->U.f);
		destroy_field(h->Unew.f);
		destroy_field(h->Ut.f);
		destroy_field(h->P.f);
	}
	delete h;
	return MESH_OK;
}

int mesh_hmc_field(mesh_hmc h, int which, mesh_field *out)
{
	return api([&] {
		require(h != nullptr && out != nullptr, "null argument");
		require(which == 0 || which == 1, "which must be 0 (U) or 1 (P)");
		*out = which == 0 ? &h->U : &h->P;
		// the caller may write through the handle: recompute S_old
		h->S_valid = false;
	});
}

int mesh_hmc_randomize(mesh_hmc h)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		DeviceGuard dg(h->ctx->device);
		ops_for(h->U.f).random(h->U.f, h->seed, 0, RedSlot{});
		h->S_valid = false;
	});
}

int mesh_hmc_cold_start(mesh_hmc h)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		DeviceGuard dg(h->ctx->device);
		ops_for(h->U.f).set_unit(h->U.f);
		h->S_valid = false;
	});
}

int mesh_hmc_save(mesh_hmc h, char const *path)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		DeviceGuard dg(h->ctx->device);
		uint64_t traj = 0;
		MESH_CUDA(cudaMemcpyAsync(&traj, &h->d_dev->traj, sizeof(traj), cudaMemcpyDeviceToHost, h->ctx->stream));
		Field const &u = h->U.f;
		std::vector<unsigned char> buf(u.host_bytes());
		export_host(u, buf.data(), buf.size()); // synchronises the stream
		config_write(path, config_header_of(u, traj, h->seed), buf.data(), buf.size());
	});
}

int mesh_hmc_load(mesh_hmc h, char const *path)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		ConfigHeader hd = config_read_header(path);
		Field &u = h->U.f;
		config_check_matches(hd, u);
		if (hd.seed != h->seed)
			throw Error(MESH_ERR_STATE, "seed mismatch on resume (the chain's streams are keyed by its seed)");
		require(hd.trajectory < uint64_t(1) << 30, "trajectory counter out of range");
		std::vector<unsigned char> buf(u.host_bytes());
		config_read_data(path, hd, buf.data(), buf.size());
		DeviceGuard dg(h->ctx->device);
		import_host(u, buf.data(), buf.size());
		int64_t traj = int64_t(hd.trajectory);
		h->ensure_history(traj + 1);
		// records before the resume point are not in the file: zero them
		MESH_CUDA(cudaMemsetAsync(h->d_hist, 0, sizeof(HmcRecordDev) * size_t(traj), h->ctx->stream));
		uint64_t t = hd.trajectory;
		MESH_CUDA(cudaMemcpyAsync(&h->d_dev->traj, &t, sizeof(t), cudaMemcpyHostToDevice, h->ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
		h->count = traj;
		h->S_valid = false;
	});
}

int mesh_hmc_momentum_step(mesh_hmc h, double beta, double delta)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		DeviceGuard dg(h->ctx->device);
		Field &U = h->U.f, &P = h->P.f;
		ops_for(U).hmc_momentum_step(P, U, beta / (2.0 * group_nc(U.group)) * delta, nullptr);
	});
}

int mesh_hmc_md_step(mesh_hmc h, double beta, double dp, double du)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		DeviceGuard dg(h->ctx->device);
		Field &U = h->U.f, &P = h->P.f;
		auto const &ops = ops_for(U);
		double coef = beta / (2.0 * group_nc(U.group)) * dp;
		if (ops.hmc_md_step(P, U, h->Ut.f, coef, du, false, nullptr))
		{
			// the new links are in Ut: swap the buffers (a captured trajectory
			// holds the old addresses, so it is dropped)
			std::swap(U.d, h->Ut.f.d);
			h->drop_graph();
		}
		else
		{
			ops.hmc_momentum_step(P, U, coef, nullptr);
			ops.hmc_evolve(U, U, P, du, false);
		}
		h->S_valid = false;
	});
}

static void copy_rec(HmcRecordDev const &r, mesh_hmc_record *rec)
{
	if (!rec)
		return;
	rec->plaquette = r.plaq;
	rec->dH = r.dH;
	rec->accept = r.accept;
	rec->H_old = r.H_old;
	rec->H_new = r.H_new;
}

int mesh_hmc_update(mesh_hmc h, double beta, double const *deltas, int n, mesh_hmc_record *rec)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		check_deltas(deltas, n);
		DeviceGuard dg(h->ctx->device);
		h->ensure_history(h->count + 1);
		int64_t k = h->count;
		h->enqueue(beta, deltas, n, nullptr, std::numeric_limits<double>::quiet_NaN());
		h->check_bad();
		copy_rec(h->record(k), rec);
	});
}

int mesh_hmc_update_supplied(mesh_hmc h, mesh_field P0, double uniform, double beta, double const *deltas, int n,
                             mesh_hmc_record *rec)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		Field &p0 = F(P0);
		same_shape(h->P.f, p0);
		require(p0.kind == MESH_ALGEBRA && p0.nstack == h->P.f.nstack, "supplied momenta must match the chain");
		require(std::isfinite(uniform), "uniform must be finite");
		check_deltas(deltas, n);
		DeviceGuard dg(h->ctx->device);
		h->ensure_history(h->count + 1);
		h->S_valid = false; // H_old from wilsonAction(U) as in hmc.cpp:85
		int64_t k = h->count;
		h->enqueue(beta, deltas, n, &p0, uniform);
		h->check_bad();
		copy_rec(h->record(k), rec);
	});
}

int mesh_hmc_run(mesh_hmc h, double beta, double const *deltas, int n, int count, int use_graph)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		check_deltas(deltas, n);
		require(count >= 0, "count must be >= 0");
		DeviceGuard dg(h->ctx->device);
		h->ensure_history(h->count + count);
		double nan = std::numeric_limits<double>::quiet_NaN();
		if (!use_graph)
		{
			for (int k = 0; k < count; ++k)
				h->enqueue(beta, deltas, n, nullptr, nan);
			return;
		}
		if (!h->S_valid)
		{
			ops_for(h->U.f).hmc_plaquette(h->U.f, h->rs(mesh_hmc_s::S_CUR));
			h->S_valid = true;
		}
		// choose launch variants before capturing (tuning times kernels)
		ops_for(h->U.f).hmc_tune(h->P.f, h->Unew.f);
		ops_for(h->U.f).hmc_tune_md(h->P.f, h->Unew.f, h->Ut.f);
		std::vector<double> dv(deltas, deltas + n);
		if (!h->graph || h->graph_beta != beta || h->graph_deltas != dv || h->graph_hist != h->d_hist)
		{
			h->drop_graph();
			cudaStream_t s = h->ctx->stream;
			cudaGraph_t g = nullptr;
			MESH_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
			int64_t saved = h->count;
			try
			{
				h->enqueue(beta, deltas, n, nullptr, nan);
			}
			catch (...)
			{
				cudaStreamEndCapture(s, &g);
				if (g)
					cudaGraphDestroy(g);
				throw;
			}
			h->count = saved;
			MESH_CUDA(cudaStreamEndCapture(s, &g));
			cudaGraphExec_t exec = nullptr;
			cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
			cudaGraphDestroy(g);
			MESH_CUDA(e);
			h->graph = exec;
			h->graph_beta = beta;
			h->graph_deltas = dv;
			h->graph_hist = h->d_hist;
		}
		for (int k = 0; k < count; ++k)
			MESH_CUDA(cudaGraphLaunch(h->graph, h->ctx->stream));
		h->count += count;
	});
}

int mesh_hmc_count(mesh_hmc h, int *n)
{
	return api([&] {
		require(h != nullptr && n != nullptr, "null argument");
		*n = int(h->count);
	});
}

int mesh_hmc_history(mesh_hmc h, int first, int count, double *plaquette, double *dH, double *accept)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		require(first >= 0 && count >= 0 && int64_t(first) + count <= h->count, "history range out of bounds");
		DeviceGuard dg(h->ctx->device);
		std::vector<HmcRecordDev> buf(static_cast<size_t>(count));
		if (count)
			MESH_CUDA(cudaMemcpyAsync(buf.data(), h->d_hist + first, sizeof(HmcRecordDev) * size_t(count),
			                          cudaMemcpyDeviceToHost, h->ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
		for (int k = 0; k < count; ++k)
		{
			if (plaquette)
				plaquette[k] = buf[size_t(k)].plaq;
			if (dH)
				dH[k] = buf[size_t(k)].dH;
			if (accept)
				accept[k] = buf[size_t(k)].accept;
		}
	});
}

int mesh_hmc_run_host(mesh_hmc h, void *host_U, size_t bytes, double beta, double const *deltas, int n, int count,
                      mesh_hmc_record *last)
{
	return api([&] {
		require(h != nullptr, "null hmc");
		require(count >= 1, "count must be >= 1");
		check_deltas(deltas, n);
		DeviceGuard dg(h->ctx->device);
		import_host(h->U.f, host_U, bytes);
		h->S_valid = false;
		h->ensure_history(h->count + count);
		double nan = std::numeric_limits<double>::quiet_NaN();
		for (int k = 0; k < count; ++k)
			h->enqueue(beta, deltas, n, nullptr, nan);
		export_host(h->U.f, host_U, bytes);
		h->check_bad();
		copy_rec(h->record(h->count - 1), last);
	});
}

// ---- Landau ------------------------------------------------------------------
static void check_landau(Field const &U, Field const &g)
{
	check_gauge(U);
	same_shape(U, g);
	require(g.kind == MESH_GROUP && g.nstack == 1, "gauge transform must be a single-component group field");
}

int mesh_landau_functional(mesh_field Uh, mesh_field gh, double *out)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		require(out != nullptr, "null output");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).landau_functional(U, g, slot(*U.ctx, SLOT_TMP));
		*out = read_slot(*U.ctx, SLOT_TMP) / (double(group_nc(U.group)) * U.nd * double(U.geom.V));
	});
}

static double landau_theta(Field const &U, Field const &g)
{
	ops_for(U).landau_theta(U, g, slot(*U.ctx, SLOT_TMP));
	double t = read_slot(*U.ctx, SLOT_TMP) / (double(U.nd) * double(U.geom.V));
	if (!std::isfinite(t))
		throw Error(MESH_ERR_NUMERIC, "non-finite gauge condition theta");
	return t;
}

int mesh_landau_theta(mesh_field Uh, mesh_field gh, double *out)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		require(out != nullptr, "null output");
		DeviceGuard dg(U.ctx->device);
		*out = landau_theta(U, g);
	});
}

int mesh_landau_deriv(mesh_field Fh, mesh_field Uh, mesh_field gh)
{
	return api([&] {
		Field &Fo = F(Fh), &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		same_shape(Fo, U);
		require(Fo.kind == MESH_ALGEBRA && Fo.nstack == 1, "output must be a single-component algebra field");
		DeviceGuard dg(U.ctx->device);
		ops_for(U).landau_deriv(Fo, U, g, -0.5 / (double(group_nc(U.group)) * U.nd * double(U.geom.V)));
	});
}

// Landau::line_search (landau.h:77-98): the step along the algebra field Fd
// from g that the three-point quadratic model of the functional puts at its
// maximum (after halving eps until the functional rises; 0 below 1e-10);
// gt is scratch for exp(eps Fd) g
static double landau_line_search(Field const &U, Field const &g, Field const &Fd, Field &gt, double eps)
{
	Context &c = *U.ctx;
	auto const &ops = ops_for(U);
	double norm_fac = 1.0 / (double(group_nc(U.group)) * U.nd * double(U.geom.V));
	auto functional = [&](Field const &h) {
		ops.landau_functional(U, h, slot(c, SLOT_TMP));
		return read_slot(c, SLOT_TMP) * norm_fac;
	};
	auto stepped = [&](double e) {
		ops.exp_apply(gt, Fd, e, g);
		return functional(gt);
	};
	double base = functional(g);
	double y1 = stepped(eps);
	while (y1 <= base)
	{
		eps *= 0.5;
		y1 = stepped(eps);
		if (eps < 1e-10)
			return 0.0;
	}
	double y2 = stepped(eps * 1.2);
	if (y2 > y1)
		return 1.2 * eps;
	double y3 = stepped(eps * 0.8);
	double x1 = eps, x2 = 1.2 * eps, x3 = 0.8 * eps;
	return 0.5 * ((x2 * x2 - x3 * x3) * y1 - (x1 * x1 - x3 * x3) * y2 + (x1 * x1 - x2 * x2) * y3) /
	       ((x2 - x3) * y1 - (x1 - x3) * y2 + (x1 - x2) * y3);
}

int mesh_landau_line_search(mesh_field Uh, mesh_field gh, mesh_field Fh, double eps, double *step)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh), &Fd = F(Fh);
		check_landau(U, g);
		require(Fd.kind == MESH_ALGEBRA && Fd.nstack == 1, "F must be a single-component algebra field");
		same_shape(U, Fd);
		require(step != nullptr && eps > 0, "invalid argument");
		Context &c = *U.ctx;
		DeviceGuard dg(c.device);
		Field gt;
		struct Cleanup
		{
			Field *a;
			~Cleanup() { destroy_field(*a); }
		} cleanup{&gt};
		create_field(c, MESH_GROUP, U.group, U.prec, U.nd, U.dims, 1, gt);
		*step = landau_line_search(U, g, Fd, gt, eps);
	});
}

int mesh_landau_cg(mesh_field Uh, mesh_field gh, int max_iter, double tol, int *iters, double *theta)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		require(max_iter >= 0, "max_iter must be >= 0");
		Context &c = *U.ctx;
		DeviceGuard dg(c.device);
		auto const &ops = ops_for(U);
		Field Fd, last, gt;
		struct Cleanup
		{
			Field *a, *b, *cc;
			~Cleanup()
			{
				destroy_field(*a);
				destroy_field(*b);
				destroy_field(*cc);
			}
		} cleanup{&Fd, &last, &gt};
		create_field(c, MESH_ALGEBRA, U.group, U.prec, U.nd, U.dims, 1, Fd);
		create_field(c, MESH_ALGEBRA, U.group, U.prec, U.nd, U.dims, 1, last);
		create_field(c, MESH_GROUP, U.group, U.prec, U.nd, U.dims, 1, gt);
		MESH_CUDA(cudaMemsetAsync(last.d, 0, last.bytes, c.stream));
		double norm_fac = 1.0 / (double(group_nc(U.group)) * U.nd * double(U.geom.V));
		double eps = 3000.0, lastNorm = 0.0, th = 0.0;
		int it = 0;
		bool converged = false;
		for (; it < max_iter; ++it)
		{
			th = landau_theta(U, g);
			if (th < tol)
			{
				converged = true;
				break;
			}
			ops.landau_deriv(Fd, U, g, -0.5 * norm_fac);
			// sum_real_trace(F*F) = -<F,F>, sum_real_trace(F*last) = -<F,last>
			ops.alg_dot(Fd, Fd, slot(c, SLOT_TMP));
			double norm = -read_slot(c, SLOT_TMP);
			ops.alg_dot(Fd, last, slot(c, SLOT_TMP));
			double fl = -read_slot(c, SLOT_TMP);
			double beta = (norm - fl) / lastNorm;
			MESH_CUDA(cudaMemcpyAsync(last.d, Fd.d, Fd.bytes, cudaMemcpyDeviceToDevice, c.stream));
			// landau.h:126-128: `last = F; F += last * beta` (last already equals F)
			if (it > 20 && beta > 0)
				ops.axpy_alg(Fd, beta, last);
			eps = landau_line_search(U, g, Fd, gt, eps);
			ops.exp_apply(gt, Fd, eps, g);
			MESH_CUDA(cudaMemcpyAsync(g.d, gt.d, g.bytes, cudaMemcpyDeviceToDevice, c.stream));
			ops.reunitize(g);
			lastNorm = norm;
		}
		if (!converged)
			th = landau_theta(U, g);
		if (iters)
			*iters = it;
		if (theta)
			*theta = th;
		if (!converged && !(th < tol))
			throw Error(MESH_ERR_NOCONV, "Landau CG did not reach the threshold within max_iter");
	});
}

int mesh_landau_or(mesh_field Uh, mesh_field gh, double omega, double tol, int max_sweeps, int check_every,
                   int *sweeps, double *theta)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		require(omega > 0 && omega < 2, "omega must be in (0, 2)");
		require(max_sweeps >= 0 && check_every >= 1, "invalid sweep counts");
		DeviceGuard dg(U.ctx->device);
		auto const &ops = ops_for(U);
		double th = landau_theta(U, g);
		int s = 0;
		while (!(th < tol) && s < max_sweeps)
		{
			for (int k = 0; k < check_every && s < max_sweeps; ++k, ++s)
			{
				ops.landau_or_half(U, g, omega, 0);
				ops.landau_or_half(U, g, omega, 1);
			}
			ops.reunit_exact(g);
			th = landau_theta(U, g);
		}
		if (sweeps)
			*sweeps = s;
		if (theta)
			*theta = th;
		if (!(th < tol))
			throw Error(MESH_ERR_NOCONV, "overrelaxation did not reach the threshold within max_sweeps");
	});
}

int mesh_gauge_transform(mesh_field Uh, mesh_field gh)
{
	return api([&] {
		Field &U = F(Uh), &g = F(gh);
		check_landau(U, g);
		DeviceGuard dg(U.ctx->device);
		ops_for(U).gauge_transform(U, g);
	});
}

} // extern "C"
