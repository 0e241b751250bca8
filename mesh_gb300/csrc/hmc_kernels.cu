// Device-side end of an HMC trajectory: the Metropolis test in FP64 on the
// device (the reference draws the uniform and decides on the host,
// src/gauge/hmc.cpp:92-99) and the accept-conditional copy of the proposal.
#include "field.cuh"
#include "rng.cuh"

#include <cmath>

namespace meshgb {

__global__ void k_metropolis(HmcDev *dev, HmcRecordDev *hist, double const *S_cur, double const *K_old,
                             double const *S_new, double const *K_new, double *S_cur_out, double beta,
                             double nplanes_V, double Nc, uint64_t seed, double uniform, int *accept_flag)
{
	if (threadIdx.x != 0 || blockIdx.x != 0)
		return;
	// wilsonAction = (1 - plaquette) * beta * Nd(Nd-1)/2 * V  (utils.h:141-146)
	double plaq_old = *S_cur / nplanes_V / Nc;
	double plaq_new = *S_new / nplanes_V / Nc;
	double H_old = (1.0 - plaq_old) * (beta * nplanes_V) + *K_old;
	double H_new = (1.0 - plaq_new) * (beta * nplanes_V) + *K_new;
	double dH = H_new - H_old;
	uint64_t traj = dev->traj;
	double u = isnan(uniform) ? metropolis_uniform(seed, traj) : uniform;
	bool finite = isfinite(H_old) && isfinite(H_new);
	bool acc = finite && (u < exp(-dH));
	if (!finite)
		dev->bad = 1;
	if (traj < uint64_t(dev->history_cap))
	{
		HmcRecordDev r;
		r.plaq = acc ? plaq_new : plaq_old;
		r.dH = dH;
		r.accept = acc ? 1.0 : 0.0;
		r.H_old = H_old;
		r.H_new = H_new;
		hist[traj] = r;
	}
	if (acc)
		*S_cur_out = *S_new;
	*accept_flag = acc ? 1 : 0;
	dev->accept_last = acc ? 1 : 0;
	dev->traj = traj + 1;
}

__global__ void k_copy_if(int const *flag, uint4 const *__restrict__ src, uint4 *__restrict__ dst, int64_t n16)
{
	if (*flag == 0)
		return;
	for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += int64_t(gridDim.x) * blockDim.x)
		dst[i] = src[i];
}

void launch_metropolis(Context &c, HmcDev *dev, HmcRecordDev *hist, double const *S_cur, double const *K_old,
                       double const *S_new, double const *K_new, double *S_cur_out, double beta, double nplanes_V,
                       double Nc, uint64_t seed, double uniform, int *accept_flag)
{
	k_metropolis<<<1, 32, 0, c.stream>>>(dev, hist, S_cur, K_old, S_new, K_new, S_cur_out, beta, nplanes_V, Nc, seed,
	                                     uniform, accept_flag);
	MESH_LAUNCH_CHECK();
}

void launch_copy_if(Context &c, void *dst, void const *src, size_t bytes, int const *flag)
{
	int64_t n16 = int64_t(bytes / 16);
	unsigned blocks = grid_for(c, n16, 256, 4);
	k_copy_if<<<blocks, 256, 0, c.stream>>>(flag, static_cast<uint4 const *>(src), static_cast<uint4 *>(dst), n16);
	MESH_LAUNCH_CHECK();
}

} // namespace meshgb
