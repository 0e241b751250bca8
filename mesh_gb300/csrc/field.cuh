// Host-side objects behind the C ABI handles, and the per-(group, precision,
// dimension) operation table that the C ABI dispatches through.
#pragma once

#include "common.cuh"
#include "layout.cuh"
#include "reduce.cuh"

#include <string>
#include <vector>

namespace meshgb {

struct Field
{
	Context *ctx = nullptr;
	int kind = MESH_GROUP; // MESH_GROUP / MESH_ALGEBRA
	int group = 0, prec = 0, nd = 0, nstack = 0;
	int32_t dims[4] = {0, 0, 0, 0};
	Geom geom{};
	int nr = 0;        // reals per object on the device
	int nr_host = 0;   // reals per object on the host (full group type)
	size_t real_bytes = 0;
	void *d = nullptr; // device storage
	size_t bytes = 0;

	size_t host_bytes() const { return size_t(nstack) * size_t(geom.V) * size_t(nr_host) * real_bytes; }
	bool same_grid(Field const &o) const
	{
		if (nd != o.nd || ctx != o.ctx)
			return false;
		for (int i = 0; i < nd; ++i)
			if (dims[i] != o.dims[i])
				return false;
		return true;
	}
};

inline int group_nr(int group) { return group == 1 ? 2 : group == 2 ? 4 : 18; }
inline int group_na(int group) { return group == 1 ? 1 : group == 2 ? 3 : 8; }
inline int group_nc(int group) { return group == 1 ? 1 : group == 2 ? 2 : 3; }

inline RedSlot slot(Context &c, int k)
{
	return {c.d_partials + size_t(k) * kMaxRedBlocks, c.d_results + k, c.d_counters + k};
}

// device-resident HMC bookkeeping
struct HmcDev
{
	uint64_t traj;   // trajectories done (momentum / Metropolis stream counter)
	int accept_last; // decision of the last trajectory
	int history_cap;
	int bad;         // set when a Hamiltonian is not finite
};
struct HmcRecordDev
{
	double plaq, dH, accept, H_old, H_new;
};

// Kinds of element-wise site operations (lattice_apply layer)
enum SiteOp
{
	SITE_MUL = 0,
	SITE_ADJ = 1,
	SITE_COPY = 2,
	SITE_EXP = 3,  // group dst = exp(algebra a)
	SITE_PROJ = 4, // algebra dst = antihermitian traceless part of group-type a
};

// Scalar-producing reduction slots (indices into the context's slots)
enum SlotId
{
	SLOT_TMP = 0,
	SLOT_TMP2 = 1,
};

struct OpsTable
{
	// fields
	void (*import_)(Field &f, void const *d_stage);
	void (*export_)(Field const &f, void *d_stage);
	void (*set_unit)(Field &f);
	void (*random)(Field &f, uint64_t seed, uint64_t counter, RedSlot kin);
	// momenta from the stream counter held on the device (HMC refresh)
	void (*random_momenta_dev)(Field &P, uint64_t seed, uint64_t const *counter_dev, RedSlot kin);
	void (*norm2)(Field const &f, RedSlot out);
	// lattice layer on single-component group fields
	void (*cshift)(Field &dst, Field const &src, int dir, int offset);
	void (*site_op)(int op, Field &dst, Field const &a, Field const *b);
	void (*sum_real_trace)(Field const &a, RedSlot out);
	// gauge
	void (*plaquette)(Field const &U, RedSlot out);
	void (*staple_sum)(Field &S, Field const &U, int mu);
	void (*wilson_deriv)(Field &F, Field const &U, int mu, double beta);
	void (*reunitize)(Field &U);
	void (*evolve)(Field const &Usrc, Field &Udst, Field const &P, double t, bool reunit);
	void (*momentum_step)(Field &P, Field const &U, double coef, RedSlot *kin);
	// Landau
	void (*landau_functional)(Field const &U, Field const &g, RedSlot out);
	void (*landau_theta)(Field const &U, Field const &g, RedSlot out);
	void (*landau_deriv)(Field &F, Field const &U, Field const &g, double scale);
	void (*landau_or_half)(Field const &U, Field &g, double omega, int parity);
	void (*reunit_exact)(Field &g);
	void (*alg_dot)(Field const &a, Field const &b, RedSlot out);
	void (*exp_apply)(Field &dst, Field const &F, double eps, Field const &g);
	void (*axpy_alg)(Field &y, double a, Field const &x);
	void (*gauge_transform)(Field &U, Field const &g);
	// pick launch variants for U's lattice ahead of a stream capture
	void (*tune)(Field &P, Field const &U);
	// the HMC trajectory's plaquette, link update, momentum step and tuning:
	// links known to be special unitary (SU(3) FP32 links are read as rows 0
	// and 1, row 2 rebuilt); the same as the generic ones otherwise
	void (*hmc_plaquette)(Field const &U, RedSlot out);
	void (*hmc_evolve)(Field const &Usrc, Field &Udst, Field const &P, double t, bool reunit);
	void (*hmc_momentum_step)(Field &P, Field const &U, double coef, RedSlot *kin);
	void (*hmc_tune)(Field &P, Field const &U);
	// the trajectory's momentum step fused with the link update after it:
	// P -= coef F(Uin), Uout = exp(tu P) Uin (reunitised when `reunit`);
	// returns false, launching nothing, where the fused kernel does not apply
	// (then the two steps run separately)
	bool (*hmc_md_step)(Field &P, Field const &Uin, Field &Uout, double coef, double tu, bool reunit, RedSlot *kin);
	void (*hmc_tune_md)(Field &P, Field const &Uin, Field &Uout);
	// Wilson loops (4D): Lout = Lprev U_dir(x + (n-1) dir); sum of the r x t loops
	void (*line_extend)(Field const &U, int dir, int n, void const *Lprev, void *Lout);
	void (*wilson_rt)(Field const &U, int r, int t, void const *S, void const *Tt, RedSlot out);
	// one heat-bath (overrelax = false) or overrelaxation sweep, checkerboard order
	void (*gauge_sweep)(Field &U, double beta, uint64_t seed, uint64_t ctr, bool overrelax);
	// layout conversion reading / writing a device-accessible host buffer directly
	void (*import_direct)(Field &f, void const *host);
	void (*export_direct)(Field const &f, void *host);
};

// autotuning registry (tune.cu): variant index per kernel/lattice key
int tuned_variant(std::string const &key);
void set_tuned_variant(std::string const &key, int variant, std::string const &report);
bool autotune_enabled();
// forced launch variant of the momentum step (-1: autotune)
int force_override();
void set_force_override(int v);
std::string tune_report();

OpsTable const *ops_u1(int prec, int nd);
OpsTable const *ops_su2(int prec, int nd);
OpsTable const *ops_su3(int prec, int nd);

inline OpsTable const &ops_for(int group, int prec, int nd)
{
	OpsTable const *t = nullptr;
	if (group == 1)
		t = ops_u1(prec, nd);
	else if (group == 2)
		t = ops_su2(prec, nd);
	else if (group == 3)
		t = ops_su3(prec, nd);
	require(t != nullptr, "unsupported (group, precision, dimension) combination");
	return *t;
}
inline OpsTable const &ops_for(Field const &f) { return ops_for(f.group, f.prec, f.nd); }

// MLP inference on device arrays (mlp.cu): y[n] = MLP(x[n][3])
void mlp_forward_device(Context &c, int n, float const *d_x, float const *d_params, int width, bool bf16, float *d_y);

// throws MESH_ERR_TIMEOUT when a kernel of the context gave up a bounded
// device-side wait (capi.cu)
void check_device_error(Context &c);

// the error message reported by mesh_last_error() (capi.cu)
void set_last_error(char const *msg);

// runs f, mapping exceptions to status codes (no exception crosses the ABI)
template <class F> int api_call(F &&f)
{
	try
	{
		f();
		return MESH_OK;
	}
	catch (Error const &e)
	{
		set_last_error(e.what());
		return e.code;
	}
	catch (std::exception const &e)
	{
		set_last_error(e.what());
		return MESH_ERR_ARG;
	}
}

// context ownership and host <-> device layout conversion through the
// context's staging buffer (capi.cu)
void ctx_retain(Context &c);
void ctx_release(Context *c);
void field_import_host(Field &f, void const *host, size_t bytes);
void field_export_host(Field const &f, void *host, size_t bytes);

// configuration files (io.cu): header of the file format
struct ConfigHeader
{
	char magic[8];
	int32_t version;
	int32_t group, precision, kind;
	int32_t nd, nstack;
	int32_t dims[4];
	uint64_t trajectory;
	uint64_t seed;
	uint64_t checksum;
};
size_t config_data_bytes(ConfigHeader const &h);
ConfigHeader config_header_of(Field const &f, uint64_t trajectory, uint64_t seed);
void config_write(char const *path, ConfigHeader h, void const *data, size_t bytes);
ConfigHeader config_read_header(char const *path);
void config_read_data(char const *path, ConfigHeader const &h, void *data, size_t bytes);
void config_check_matches(ConfigHeader const &h, Field const &f);

// HMC trajectory kernels (hmc.cu)
void launch_metropolis(Context &c, HmcDev *dev, HmcRecordDev *hist, double const *S_cur, double const *K_old,
                       double const *S_new, double const *K_new, double *S_cur_out, double beta, double nplanes_V,
                       double Nc, uint64_t seed, double uniform, int *accept_flag);
void launch_copy_if(Context &c, void *dst, void const *src, size_t bytes, int const *flag);

} // namespace meshgb

// objects behind the C ABI handles
struct mesh_ctx_s
{
	meshgb::Context c;
};
struct mesh_field_s
{
	meshgb::Field f;
};
