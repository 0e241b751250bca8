/*
 * mesh_gb300 — C ABI of the GB300 (sm_103a) lattice-gauge hot path.
 *
 * Drop-in boundary for krox/mesh's lattice_apply/reduction layer
 * (src/lattice), pure-gauge HMC (src/gauge/utils.h, hmc.h, hmc.cpp) and
 * Landau gauge fixing (src/gauge/landau.h). The reference exposes header
 * templates (Lattice<T>, GaugeField<G>, Hmc<G>, Landau<G>) and throws
 * std::runtime_error on CUDA errors (src/lattice/device.cpp:11-18); here every
 * entry point returns an int status (0 = MESH_OK) and never throws. The C++
 * wrapper include/mesh/mesh.hpp restores the reference's class names and
 * rethrows non-zero statuses as std::runtime_error.
 *
 * Conventions
 *  - group: MESH_U1, MESH_SU2, MESH_SU3 and precision MESH_F32 (float),
 *    MESH_F64 (double) are dispatchByGroup's runtime choices
 *    (src/gauge/utils.h:156-186; precision 1 = float, 2 = double).
 *  - Host buffers use the reference's host layout: sites lexicographic with
 *    dimension 0 slowest (src/lattice/grid.h:39-49), one block of V objects
 *    per stacked component mu (LatticeStack, src/lattice/lattice.h:159-192),
 *    objects as complex (re,im), quaternion (re,im1,im2,im3) or row-major
 *    3x3 complex matrices. Momenta/forces are algebra fields: on the host they
 *    are full group-type objects (as the reference stores them); on the
 *    device they are packed (1/3/8 reals).
 *  - Device storage is even/odd checkerboard, structure-of-arrays
 *    (mesh_field_device_ptr documents nothing more: treat it as opaque).
 *  - All extents must be even and below 256, 2 <= nd <= 4, volume < 2^31.
 *  - Calls are issued on the context's stream. Functions returning a host
 *    scalar synchronise that stream (as the reference's reductions do,
 *    src/lattice/device.h:259-260); the others are asynchronous.
 *  - Not thread-safe per context (like the reference's globals).
 */
#ifndef MESH_GB300_H
#define MESH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MESH_OK 0
#define MESH_ERR_ARG 1         /* invalid argument (shape, group, size, kind) */
#define MESH_ERR_CUDA 2        /* CUDA runtime error (device.cpp:11-18 analogue) */
#define MESH_ERR_STATE 3       /* objects on different grids/contexts, wrong state */
#define MESH_ERR_TIMEOUT 4     /* a bounded device-side wait expired (the launch's results are invalid) */
#define MESH_ERR_NUMERIC 5     /* NaN/Inf in an action, Hamiltonian or theta */
#define MESH_ERR_NOCONV 6      /* iteration limit reached without convergence */
#define MESH_ERR_UNSUPPORTED 7 /* valid request this build does not implement */

#define MESH_U1 1
#define MESH_SU2 2
#define MESH_SU3 3
#define MESH_F32 1
#define MESH_F64 2

#define MESH_GROUP 0   /* field of group elements (links, gauge transforms) */
#define MESH_ALGEBRA 1 /* field of algebra elements (momenta, forces) */

typedef struct mesh_ctx_s *mesh_ctx;
typedef struct mesh_field_s *mesh_field;
typedef struct mesh_hmc_s *mesh_hmc;
typedef struct mesh_landau_fa_s *mesh_landau_fa;

/* ---- library ------------------------------------------------------------ */
/* last error message of the calling thread (valid until the next call) */
const char *mesh_last_error(void);
/* ABI version: major*10000 + minor*100 + patch */
int mesh_version(void);

/* Autotuner report: one line per tuned kernel/lattice key with the chosen
 * launch variant and the measured candidates. Writes at most cap bytes
 * (NUL-terminated) and returns the size needed. Tuning runs once per key and
 * process, on the first call outside a stream capture; MESH_AUTOTUNE=0 in the
 * environment disables it (default variants). */
size_t mesh_tune_report(char *buf, size_t cap);
/* Forces launch variant `variant` of the fused momentum-step kernel for all
 * later calls where it is valid for the lattice (-1 restores autotuning).
 * For testing every variant against the oracle. */
int mesh_tune_force_variant(int variant);

/* ---- context: device + stream + reduction scratch ------------------------
 * Replaces the reference's implicit "current device, default stream"
 * (src/lattice/device.h:219-228). stream == NULL: the context creates and
 * owns a non-blocking stream. */
int mesh_ctx_create(int device, void *stream, mesh_ctx *out);
int mesh_ctx_destroy(mesh_ctx ctx);
int mesh_ctx_synchronize(mesh_ctx ctx);
/* the cudaStream_t the context launches on */
void *mesh_ctx_stream(mesh_ctx ctx);
/* Test of the bounded device-side waits (no reference counterpart): one
 * thread waits up to `seconds` (<= 2) for a device flag that is set before
 * the launch when flag_set != 0 and never otherwise; an expired wait is
 * recorded in the context's device error word and returned as
 * MESH_ERR_TIMEOUT, as the kernels with bounded waits report theirs. The
 * context stays usable. Synchronises the context's stream. */
int mesh_ctx_wait_probe(mesh_ctx ctx, double seconds, int flag_set);

/* ---- fields: Lattice<T> / LatticeStack<T> / GaugeField<G> ---------------
 * Replaces Lattice<T>(Grid) and LatticeStack<T>(Grid)
 * (src/lattice/lattice.h:43-47,171-176; GaugeField = LatticeStack,
 * src/gauge/utils.h:21). nstack = number of stacked components (nd for a
 * gauge field or momenta, 1 for a single Lattice). Contents are
 * uninitialised, as in the reference. */
int mesh_field_create(mesh_ctx ctx, int kind, int group, int precision, int nd, const int32_t *dims, int nstack,
                      mesh_field *out);
int mesh_field_destroy(mesh_field f);
int mesh_field_info(mesh_field f, int *kind, int *group, int *precision, int *nd, int32_t *dims, int *nstack);
/* size in bytes of the field in the reference's host layout */
size_t mesh_field_host_bytes(mesh_field f);
/* Lattice::copy_from_host / copy_to_host (lattice.h:102-115), for every
 * stacked component; the layout conversion is a bit-exact permutation. */
int mesh_field_import(mesh_field f, const void *host, size_t bytes);
int mesh_field_export(mesh_field f, void *host, size_t bytes);
/* Configuration files: the dataset writeToFile/readFromFile store
 * ([nstack][sites lexicographic][reals], lattice.h:205-252) behind a 72-byte
 * header (magic "MESHCFG1", version, group, precision, kind, nd, nstack,
 * dims[4], trajectory, seed, checksum; little-endian). Loading refuses a file
 * whose group, precision or grid differ from the field, as readConfig does
 * (utils.h:188-219), with MESH_ERR_STATE; a corrupt file (checksum) also
 * gives MESH_ERR_STATE. */
int mesh_field_save(mesh_field f, const char *path);
int mesh_field_load(mesh_field f, const char *path);
/* header of a configuration file (any output may be NULL; dims gets nd values) */
int mesh_config_info(const char *path, int *kind, int *group, int *precision, int *nd, int32_t *dims, int *nstack,
                     uint64_t *trajectory, uint64_t *seed);
/* deep copy (Lattice copy assignment, lattice.h:83-93); same shape required */
int mesh_field_copy(mesh_field dst, mesh_field src);
/* Lattice::zeros / fill_zeros (lattice.h:51-58) */
int mesh_field_set_zero(mesh_field f);
/* group fields: every element = identity (cold start; the reference's
 * Landau::reset g.fill(G(1)), landau.h:14) */
int mesh_field_set_unit(mesh_field f);
/* group fields: Haar-random elements (random_gauge_field, utils.h:43-70);
 * algebra fields: Gaussian momenta with tr(T^aT^b)=delta/2
 * (random_algebra_field, utils.h:54-78). Drawn on the device from a
 * counter-based stream (seed, counter); no host RNG, no H2D copy. */
int mesh_field_random(mesh_field f, uint64_t seed, uint64_t counter);
/* opaque device storage (even/odd structure of arrays) */
void *mesh_field_device_ptr(mesh_field f);

/* ---- lattice_apply layer on single-component group fields ----------------
 * The named site-wise operations the gauge code builds from lattice_apply
 * (src/lattice/lattice.h:256-364, src/gauge/utils.h:28-33). */
/* dst[x] = src[x + offset * e_dir], periodic (cshift, lattice.h:366-389) */
int mesh_site_cshift(mesh_field dst, mesh_field src, int dir, int offset);
/* dst = a * b (MESH_DEFINE_LATTICE_BINARY(*), lattice.h:289-301) */
int mesh_site_mul(mesh_field dst, mesh_field a, mesh_field b);
/* out = a x + b y object by object, for fields of one shape (any kind and
 * stack size); y may be NULL (out = a x), out may be x or y. Every field kind
 * stores its objects linearly (matrices, quaternions, complex numbers, packed
 * algebra), so this is the reference's lattice +, -, scalar * and their
 * compound forms (MESH_DEFINE_LATTICE_BINARY, lattice.h:289-327,337-338;
 * operator*(Lattice, double), lattice.h:348-356) and add_mul (lattice.h:358-364) */
int mesh_field_axpby(mesh_field out, double a, mesh_field x, double b, mesh_field y);
/* dst = exp(a), a an algebra field, dst a group field
 * (MESH_DEFINE_LATTICE_UNARY(exp, gauge::exp), utils.h:32) */
int mesh_site_exp(mesh_field dst, mesh_field a);
/* dst = project_on_algebra(a): the antihermitian traceless part of the
 * group-type objects of a, into an algebra field (utils.h:33;
 * groups.h:64-67,142-145,224-228) */
int mesh_site_project(mesh_field dst, mesh_field a);
/* dst = adj(a) (utils.h:31) */
int mesh_site_adj(mesh_field dst, mesh_field a);
/* sum_x real_trace(a(x)) in FP64 (sum_real_trace, utils.h:29) */
int mesh_site_sum_real_trace(mesh_field a, double *out);
/* sum of norm2 over every component (norm2(LatticeStack), utils.h:35-41);
 * algebra fields use the kinetic (defining-representation Frobenius) norm */
int mesh_field_norm2(mesh_field a, double *out);

/* ---- gauge utilities (src/gauge/utils.h) --------------------------------- */
/* plaquette normalised to [0,1] (utils.h:94-108); FP64 accumulation */
int mesh_plaquette(mesh_field U, double *out);
/* Wilson action (1 - plaquette) * beta * Nd(Nd-1)/2 * V (utils.h:141-146) */
int mesh_wilson_action(mesh_field U, double beta, double *out);
/* One heat-bath sweep of the Wilson action at beta over every link: the
 * legacy WilsonAction<G>::sweep (src/old/wilson.cpp:15-60) and
 * GaugeAction<G>::thermalize (src/old/mesh/gauge_action.h:42-56). U(1) and
 * SU(2) links are drawn from their conditional distribution given the staple
 * sum; SU(3) links by three SU(2) subgroup heat-baths (Cabibbo-Marinari).
 * Links are updated in checkerboard order (per direction, even then odd
 * sites); the random numbers are Philox draws addressed by (seed, site,
 * direction, subgroup, attempt) with counter = sweep, so a sweep number
 * replays the same update. */
int mesh_heatbath_sweep(mesh_field U, double beta, uint64_t seed, uint64_t sweep);
/* One overrelaxation sweep: every link reflected so that ReTr(U S) with its
 * staple sum S is unchanged (GaugeAction<G>::overrelax,
 * src/old/mesh/gauge_action.h:59-73; SU(3) through its three SU(2) subgroups,
 * where the legacy formula would not keep the action). The action is
 * unchanged up to rounding. */
int mesh_overrelax_sweep(mesh_field U);
/* Rectangular Wilson loops W(r, t) for r = 1..max_r, t = 1..max_t in the planes
 * (mu, 3), mu = 0, 1, 2: the legacy wilson() of src/old/mesh/wilson.cpp:40-75
 * (spatial line of r links, temporal line of t links, averaged over sites and
 * the three spatial directions), normalised like the plaquette (ReTr / Nc, so
 * W(1, 1) is the mean plaquette of the planes (mu, 3)). out[(r-1) max_t + t-1].
 * 4D lattices; max_r <= min(L0, L1, L2), max_t <= L3. Allocates (max_t + 3)
 * link components of scratch for the call. */
int mesh_wilson_loops(mesh_field U, int max_r, int max_t, double *out);

/* Plaquette without any device allocation. No counterpart in the reference.
 * For callers that cannot call cudaMalloc when they measure: applications
 * that give all device memory to their own pool or arena at start-up and
 * forbid later allocations, or that run under a memory cap where a context
 * (mesh_ctx_create allocates reduction scratch, a stream and staging) cannot
 * be made. They pass plain pointers: `links` is a device buffer on `device`
 * holding a gauge field of (group, precision, nd, dims) in the library's
 * device storage (what mesh_field_device_ptr returns for such a field).
 * Same kernel and grid as mesh_plaquette, so the same value bit for bit.
 * Its reduction scratch is a static device array inside the library of
 * MESH_NOALLOC_MAX_BLOCKS partial sums (8 KiB); a launch that would need more
 * blocks is refused with MESH_ERR_ARG (none does on devices of up to 256 SMs).
 * `links` is checked with cudaPointerGetAttributes (no allocation): host
 * memory or another device's buffer is refused with MESH_ERR_ARG before
 * anything is launched.
 * The first call on a device does set-up (may create the device's primary
 * context and load the library's kernels, then resolves the scratch
 * address); make that call before any stream capture. A set-up that fails
 * returns MESH_ERR_CUDA and is tried again by the next call. Every call
 * runs on `stream` (NULL: the legacy default stream) and waits for it: the
 * result is read back to the host before the function returns. The scratch
 * is shared by all callers in the process: calls that overlap on one device
 * (several host threads, or work still in flight on another stream) race and
 * must be serialised by the caller. */
#define MESH_NOALLOC_MAX_BLOCKS 1024
int mesh_plaquette_noalloc(int device, int group, int precision, int nd, const int32_t *dims, const void *links,
                           void *stream, double *out);
/* S = staple sum for direction mu (stapleSum, utils.h:114-139); S is a
 * single-component group field on U's grid */
int mesh_staple_sum(mesh_field S, mesh_field U, int mu);
/* F = project_on_algebra(U_mu * S_mu * beta / (2 Nc)) (wilsonDeriv,
 * utils.h:148-153); F is a single-component algebra field */
int mesh_wilson_deriv(mesh_field F, mesh_field U, int mu, double beta);
/* project_on_group_fast on every link (reunitize, utils.h:80-91) */
int mesh_reunitize(mesh_field U);

/* ---- HMC building blocks (src/gauge/hmc.h, hmc.cpp) ---------------------- */
/* U_mu <- exp(project_on_algebra(P_mu) * t) U_mu for all mu (evolve,
 * hmc.h:26-36) */
int mesh_evolve(mesh_field U, mesh_field P, double t);
/* P_mu -= wilsonDeriv(U, mu, beta) * delta for all mu (the momentum step
 * of runHmd, hmc.h:54-58), fused: staples, product, projection and update
 * in one kernel */
int mesh_momentum_step(mesh_field P, mesh_field U, double beta, double delta);
/* runHmd (hmc.h:38-59): alternating position/momentum steps */
int mesh_run_hmd(mesh_field U, mesh_field P, double beta, const double *deltas, int n);
/* makeDeltas (hmc.cpp:7-51): scheme "2lf", "2mn" or "4mn"; writes at most
 * capacity values and the count to *n */
int mesh_make_deltas(const char *scheme, double epsilon, int substeps, double *out, int capacity, int *n);

/* ---- HMC chain: Hmc<G> (hmc.h:66-115, hmc.cpp:56-106) ------------------
 * Owns U, P and the proposal U_new. Momenta and the Metropolis uniform come
 * from counter-based device streams keyed by `seed` and the trajectory
 * number; H_old/H_new, dH and the accept decision are computed on the device
 * in FP64. */
typedef struct mesh_hmc_record
{
	double plaquette; /* plaquette(U) after the accept/reject step */
	double dH;        /* H_new - H_old */
	double accept;    /* 1.0 accepted, 0.0 rejected */
	double H_old, H_new;
} mesh_hmc_record;

int mesh_hmc_create(mesh_ctx ctx, int group, int precision, int nd, const int32_t *dims, uint64_t seed,
                    mesh_hmc *out);
int mesh_hmc_destroy(mesh_hmc h);
/* borrowed handles of the state: which = 0 -> U, 1 -> P */
int mesh_hmc_field(mesh_hmc h, int which, mesh_field *out);
/* randomizeGaugeField (hmc.cpp:58-62) and a cold start */
int mesh_hmc_randomize(mesh_hmc h);
int mesh_hmc_cold_start(mesh_hmc h);
/* Checkpoint and resume: U, the trajectory counter and the seed in a
 * configuration file. A chain with the same seed that loads it continues
 * exactly as the saved chain would have (same momentum and Metropolis
 * streams); records before the resume point read as zero. */
int mesh_hmc_save(mesh_hmc h, const char *path);
int mesh_hmc_load(mesh_hmc h, const char *path);
/* One momentum step P -= beta/(2 Nc) delta proj(U S) on the chain's own U
 * and P with the trajectory's kernel (SU(3) FP32 links read as rows 0 and 1,
 * row 2 rebuilt; the autotuned launch variant): for timing and tests. */
int mesh_hmc_momentum_step(mesh_hmc h, double beta, double delta);
/* One momentum step of size dp followed by one link update of size du on the
 * chain's own U and P: the inner pair of runHmd (hmc.h:38-59), i.e.
 * P -= beta/(2 Nc) dp proj(U S), then U <- exp(du P) U (evolve, hmc.h:26-36).
 * With FP32 fields on a lattice the thread-per-site kernel tiles, both run in
 * the one fused kernel the trajectory uses (the links are written out of
 * place and the chain's buffers swapped); otherwise as two kernels. */
int mesh_hmc_md_step(mesh_hmc h, double beta, double dp, double du);
/* runHmcUpdate (hmc.cpp:73-107): one trajectory, synchronous, record out */
int mesh_hmc_update(mesh_hmc h, double beta, const double *deltas, int n, mesh_hmc_record *rec);
/* One trajectory on caller-supplied momenta P0 (algebra field, copied, not
 * modified) and Metropolis uniform: the parity entry point. */
int mesh_hmc_update_supplied(mesh_hmc h, mesh_field P0, double uniform, double beta, const double *deltas, int n,
                             mesh_hmc_record *rec);
/* `count` trajectories without host synchronisation. use_graph != 0
 * captures one trajectory in a CUDA graph and replays it. Records go to a
 * device history read by mesh_hmc_history. */
int mesh_hmc_run(mesh_hmc h, double beta, const double *deltas, int n, int count, int use_graph);
/* number of trajectories recorded so far */
int mesh_hmc_count(mesh_hmc h, int *n);
/* copy records [first, first+count) to host arrays (any may be NULL) */
int mesh_hmc_history(mesh_hmc h, int first, int count, double *plaquette, double *dH, double *accept);
/* HMC with the gauge field exchanged in the reference's host layout every
 * call: import U from host, run `count` trajectories, export U to host. */
int mesh_hmc_run_host(mesh_hmc h, void *host_U, size_t bytes, double beta, const double *deltas, int n, int count,
                      mesh_hmc_record *last);

/* ---- batched replicas (no reference counterpart) --------------------------
 * Many independent 4D lattices of one group and precision, each with its own
 * extents, beta and seed, advanced together: every step of the trajectory
 * sequence of runHmcUpdate (hmc.cpp:73-107) is one persistent launch over
 * all replicas. Replica r follows the trajectory of a single chain
 * (mesh_hmc_*) created with seeds[r]: same momentum and Metropolis streams,
 * same per-link arithmetic. */
typedef struct mesh_batch_s *mesh_batch;
/* dims: nrep x 4 extents (even, < 256); seeds: nrep keys. Links start as unit. */
int mesh_batch_create(mesh_ctx ctx, int group, int precision, int nrep, const int32_t *dims, const uint64_t *seeds,
                      mesh_batch *out);
int mesh_batch_destroy(mesh_batch h);
int mesh_batch_size(mesh_batch h, int *nrep);
/* Haar-random links (each replica as mesh_hmc_randomize with its seed) / unit links */
int mesh_batch_randomize(mesh_batch h);
int mesh_batch_cold_start(mesh_batch h);
/* replica r's links in the reference's host layout (mesh_field_import/export) */
int mesh_batch_import(mesh_batch h, int r, const void *host, size_t bytes);
int mesh_batch_export(mesh_batch h, int r, void *host, size_t bytes);
/* `count` trajectories of every replica, betas[r] per replica; use_graph != 0
 * replays one captured trajectory of the whole batch. Synchronous. */
int mesh_batch_run(mesh_batch h, const double *betas, const double *deltas, int n, int count, int use_graph);
int mesh_batch_count(mesh_batch h, int *n);
/* replica r's records [first, first+count) (any output may be NULL) */
int mesh_batch_history(mesh_batch h, int r, int first, int count, double *plaquette, double *dH, double *accept);
/* plaquette of every replica's current links (nrep values) */
int mesh_batch_plaquettes(mesh_batch h, double *out);
/* kernel launches per trajectory for an n_deltas-step table, and the
 * persistent grids of the link and site kernels (any output may be NULL) */
int mesh_batch_launch_info(mesh_batch h, int *launches_per_trajectory, int n_deltas, int *grid_links,
                           int *grid_sites);
/* the MD-step form the first run timed and chose: fused = 1 (momentum step
 * and link update in one kernel) or 0 (separate kernels), -1 before the first
 * run; the fused kernel's launch variant, its minimum resident blocks per SM
 * (the register cap it was compiled under) and its persistent grid (any
 * output may be NULL). No reference counterpart: the batch is new. */
int mesh_batch_md_launch(mesh_batch h, int *fused, int *variant, int *min_blocks, int *grid);

/* ---- Landau gauge fixing (src/gauge/landau.h) ----------------------------
 * g is a single-component group field (the gauge transform); U is not
 * modified. */
/* functional sum_mu sum_x ReTr(g(x) U_mu(x) g(x+mu)^dagger)/(Nc Nd V)
 * (Landau::operator(), landau.h:23-32), FP64 */
int mesh_landau_functional(mesh_field U, mesh_field g, double *out);
/* Landau::line_search (landau.h:77-98): the step along the algebra field F
 * (single component) from g that mesh_landau_cg takes (halving eps until
 * the functional rises, then the quadratic model through eps, 1.2 eps,
 * 0.8 eps; 0 when eps falls below 1e-10) */
int mesh_landau_line_search(mesh_field U, mesh_field g, mesh_field F, double eps, double *step);
/* theta_ref = sum_x |Delta(x)|^2 / (Nd V), Delta = sum_mu A_mu(x)-A_mu(x-mu)
 * (Landau::condition, landau.h:37-49), FP64 */
int mesh_landau_theta(mesh_field U, mesh_field g, double *out);
/* F = project_on_algebra(g d) * (-0.5/(Nc Nd V)) (Landau::deriv,
 * landau.h:52-65); F a single-component algebra field */
int mesh_landau_deriv(mesh_field F, mesh_field U, mesh_field g);
/* the reference's nonlinear CG with line search (Landau::run,
 * landau.h:100-136) with the stopping threshold as an argument */
int mesh_landau_cg(mesh_field U, mesh_field g, int max_iter, double tol, int *iters, double *theta);
/* checkerboard overrelaxation (no reference counterpart; the legacy
 * relaxation of src/old/gauge_fixing.cpp:33-79 overrelaxed): sweeps in
 * blocks of check_every, theta_ref after each block, stop below tol */
int mesh_landau_or(mesh_field U, mesh_field g, double omega, double tol, int max_sweeps, int check_every,
                   int *sweeps, double *theta);
/* U <- g U g^dagger(x+mu) for all mu (apply a gauge transform) */
int mesh_gauge_transform(mesh_field U, mesh_field g);

/* ---- Fourier-accelerated Landau gauge fixing (no reference counterpart;
 * the reference's FFT helpers, src/lattice/fft.h:36-61, wrap FFTW on the host
 * and are unused) -------------------------------------------------------------
 * Steepest descent with a spectral multiplier (Davies et al., Phys. Rev. D 37
 * (1988) 1581): g <- reunit(exp(-F^-1[m(p) F[Delta]]/V) g), Delta the lattice
 * divergence of the gauge-fixed links. g and U are FP64; the transform is an
 * FP32 FFT (it only shapes the step); theta is FP64. Extents must be
 * 2,4,6,8,12,16,24 or 32. The workspace borrows U (keep it alive). */
int mesh_landau_fa_create(mesh_field U, mesh_landau_fa *out);
int mesh_landau_fa_destroy(mesh_landau_fa h);
/* m(p) = alpha * p2max / phat^2(p), 0 at p = 0 (phat^2 = sum 4 sin^2(pi n/L)) */
int mesh_landau_fa_set_plain(mesh_landau_fa h, double alpha);
/* m(p) = exp(table) sampled on n points uniform in log phat^2 */
int mesh_landau_fa_set_table(mesh_landau_fa h, const float *log_mult, int n, double log_p2_lo, double log_p2_hi);
/* learned multiplier: log m = MLP(log phat^2 - log p2max, 5(beta-6),
 * (log10 theta + 7)/5), width 32 or 64, re-evaluated before every step
 * (BF16 inference when bf16 != 0) */
int mesh_landau_fa_set_mlp(mesh_landau_fa h, const float *params, int width, double beta, int bf16);
/* smallest non-zero and largest phat^2 of the lattice */
int mesh_landau_fa_p2range(mesh_landau_fa h, double *p2min, double *p2max);
/* theta_ref of g (FP64) */
int mesh_landau_fa_theta(mesh_landau_fa h, mesh_field g, double *theta);
/* one step in place; theta of g before the step */
int mesh_landau_fa_step(mesh_landau_fa h, mesh_field g, double *theta_before);
/* steps until theta < tol; a step that does not lower theta is undone and
 * or_sweeps overrelaxation sweeps (omega) run instead (the fallback). With
 * mesh_landau_fa_set_accept(h, 1) the test is on the gauge functional
 * instead: a step is undone when it lowered sum Re tr g U g^+ by more than
 * its FP64 summation error (theta, the norm of the gradient, may rise for a
 * step while the functional rises) */
int mesh_landau_fa_run(mesh_landau_fa h, mesh_field g, double tol, int max_iter, double omega, int or_sweeps,
                       int *iters, int *fallbacks, double *theta);
/* acceptance test of mesh_landau_fa_run: 0 = theta (default), 1 = the gauge functional */
int mesh_landau_fa_set_accept(mesh_landau_fa h, int on_functional);
/* trial step that leaves g unchanged (the current multiplier, or the plain
 * one with alpha when alpha > 0): theta before and after */
int mesh_landau_fa_trial(mesh_landau_fa h, mesh_field g, double alpha, double *theta_before, double *theta_after);
/* response of the momentum modes to a probe step (multiplier probe_alpha
 * p2max/phat^2), per bin of log phat^2: mean phat^2, lambda = effective
 * contraction rate per unit multiplier, weight, count; theta of g */
int mesh_landau_fa_probe(mesh_landau_fa h, mesh_field g, double probe_alpha, int nbins, double *p2_mean,
                         double *lambda, double *weight, double *count, double *theta);

/* ---- lattice FFT (fft_all, src/lattice/fft.h:55-58) ----------------------------
 * unnormalised FFT over every axis of nf complex FP32 fields, host array
 * [nf][V] interleaved (re, im), lexicographic sites; sign -1 forward
 * (e^{-2 pi i k x/L}), +1 backward */
int mesh_lattice_fft(mesh_ctx ctx, int nd, const int32_t *dims, int nf, float *data, int sign);

/* ---- the learned multiplier's network (3 -> width -> width -> 1 tanh MLP) --
 * params (float): W1[w][3] b1[w] W2[w][w] b2[w] W3[w] b3; host arrays;
 * computed on the context's device */
int mesh_mlp_nparams(int width);
int mesh_mlp_forward(mesh_ctx ctx, int n, const float *x, const float *params, int width, int bf16, float *y);
/* mean squared error over n samples and its gradient (backward pass) */
int mesh_mlp_grad(mesh_ctx ctx, int n, const float *x, const float *t, const float *params, int width, double *loss,
                  float *grad);
/* Adam training in shuffled minibatches, params updated in place */
int mesh_mlp_train(mesh_ctx ctx, int n, const float *x, const float *t, float *params, int width, int epochs,
                   int batch, float lr, uint64_t seed, float *loss_per_epoch);

#ifdef __cplusplus
}
#endif

#endif /* MESH_GB300_H */
