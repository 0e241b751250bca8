// The learned spectral multiplier of Fourier-accelerated Landau gauge fixing:
// a 3-layer tanh MLP 3 -> W -> W -> 1 (W = 64), FP32 weights.
//   h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), y = W3 . h2 + b3
// Parameter layout (float): W1[W][3] b1[W] W2[W][W] b2[W] W3[W] b3.
// Kernels: FP32 forward, BF16 inference (bf16 weights and activations, FP32
// accumulation), mean-squared-error loss with its gradient (backward pass),
// Adam update; host entry points for inference, the gradient (checked
// against the CPU oracle's FP64 backward pass) and a full training loop.
#include "field.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <vector>

using namespace meshgb;

namespace {

constexpr int nparams(int w) { return 3 * w + w + w * w + w + w + 1; }

template <int W> struct Off
{
	static constexpr int W1 = 0, B1 = 3 * W, W2 = B1 + W, B2 = W2 + W * W, W3 = B2 + W, B3 = W3 + W, N = B3 + 1;
};

// ---- inference: one thread per sample, weights in shared memory -------------
template <int W, bool BF16>
__global__ void __launch_bounds__(128) k_mlp_forward(int n, float const *__restrict__ x,
                                                     float const *__restrict__ params, float *__restrict__ y)
{
	using O = Off<W>;
	extern __shared__ unsigned char smraw[];
	float *sw = reinterpret_cast<float *>(smraw);
	__nv_bfloat16 *sb = reinterpret_cast<__nv_bfloat16 *>(smraw);
	for (int i = threadIdx.x; i < O::N; i += blockDim.x)
	{
		if constexpr (BF16)
			sb[i] = __float2bfloat16(params[i]);
		else
			sw[i] = params[i];
	}
	__syncthreads();
	auto P = [&](int i) -> float {
		if constexpr (BF16)
			return __bfloat162float(sb[i]);
		else
			return sw[i];
	};
	auto act = [&](float v) -> float {
		float t = tanhf(v);
		if constexpr (BF16)
			return __bfloat162float(__float2bfloat16(t));
		else
			return t;
	};
	for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
	{
		float xi[3];
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			xi[k] = x[3 * s + k];
			if constexpr (BF16)
				xi[k] = __bfloat162float(__float2bfloat16(xi[k]));
		}
		float h1[W];
#pragma unroll
		for (int i = 0; i < W; ++i)
			h1[i] = act(P(O::B1 + i) + P(O::W1 + 3 * i) * xi[0] + P(O::W1 + 3 * i + 1) * xi[1] +
			            P(O::W1 + 3 * i + 2) * xi[2]);
		float out = P(O::B3);
#pragma unroll 4
		for (int i = 0; i < W; ++i)
		{
			float a = P(O::B2 + i);
#pragma unroll
			for (int k = 0; k < W; ++k)
				a += P(O::W2 + W * i + k) * h1[k];
			out += P(O::W3 + i) * act(a);
		}
		y[s] = out;
	}
}

// ---- gradient: a block of W threads, thread i owns hidden unit i ------------
// Each block processes samples idx[b0 .. b1) (a chunk of the batch) one at a
// time; thread i keeps row i of W2 and of its gradient in registers; the
// gradient of the chunk is added to `grad` with one atomic per parameter.
template <int W>
__global__ void __launch_bounds__(W) k_mlp_grad(int n_batch, int const *__restrict__ idx, float const *__restrict__ x,
                                                float const *__restrict__ t, float const *__restrict__ params,
                                                int chunk, float inv_n, float *__restrict__ grad,
                                                double *__restrict__ loss)
{
	using O = Off<W>;
	__shared__ float sW2[W * W];
	__shared__ float sh1[W], sd2[W], sred[W / 32];
	__shared__ float sdy;
	int i = threadIdx.x;
	for (int k = i; k < W * W; k += W)
		sW2[k] = params[O::W2 + k];
	float w1[3] = {params[O::W1 + 3 * i], params[O::W1 + 3 * i + 1], params[O::W1 + 3 * i + 2]};
	float b1 = params[O::B1 + i], b2 = params[O::B2 + i], w3 = params[O::W3 + i], b3 = params[O::B3];
	float w2row[W];
#pragma unroll
	for (int k = 0; k < W; ++k)
		w2row[k] = params[O::W2 + W * i + k];
	float gW2[W];
#pragma unroll
	for (int k = 0; k < W; ++k)
		gW2[k] = 0.f;
	float gW1[3] = {0.f, 0.f, 0.f}, gb1 = 0.f, gb2 = 0.f, gW3 = 0.f, gb3 = 0.f;
	double lsum = 0.0;
	__syncthreads();
	int b0 = blockIdx.x * chunk, b1e = min(n_batch, b0 + chunk);
	for (int b = b0; b < b1e; ++b)
	{
		int s = idx ? idx[b] : b;
		float x0 = x[3 * s], x1 = x[3 * s + 1], x2 = x[3 * s + 2];
		float h1 = tanhf(b1 + w1[0] * x0 + w1[1] * x1 + w1[2] * x2);
		sh1[i] = h1;
		__syncthreads();
		float a2 = b2;
#pragma unroll
		for (int k = 0; k < W; ++k)
			a2 += w2row[k] * sh1[k];
		float h2 = tanhf(a2);
		// y = b3 + sum_i w3_i h2_i
		float part = w3 * h2;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
			part += __shfl_down_sync(0xffffffffu, part, o);
		if ((i & 31) == 0)
			sred[i >> 5] = part;
		__syncthreads();
		if (i == 0)
		{
			float yv = b3;
#pragma unroll
			for (int wv = 0; wv < W / 32; ++wv)
				yv += sred[wv];
			float e = yv - t[s];
			lsum += double(e) * double(e);
			sdy = 2.f * e * inv_n;
		}
		__syncthreads();
		float dy = sdy;
		gb3 += dy;
		gW3 += dy * h2;
		float d2 = dy * w3 * (1.f - h2 * h2);
		gb2 += d2;
#pragma unroll
		for (int k = 0; k < W; ++k)
			gW2[k] += d2 * sh1[k];
		sd2[i] = d2;
		__syncthreads();
		// d1_i = (sum_j d2_j W2[j][i]) (1 - h1_i^2)
		float a = 0.f;
#pragma unroll
		for (int j = 0; j < W; ++j)
			a += sd2[j] * sW2[W * j + i];
		float d1 = a * (1.f - h1 * h1);
		gb1 += d1;
		gW1[0] += d1 * x0;
		gW1[1] += d1 * x1;
		gW1[2] += d1 * x2;
		__syncthreads();
	}
	atomicAdd(grad + O::W1 + 3 * i, gW1[0]);
	atomicAdd(grad + O::W1 + 3 * i + 1, gW1[1]);
	atomicAdd(grad + O::W1 + 3 * i + 2, gW1[2]);
	atomicAdd(grad + O::B1 + i, gb1);
#pragma unroll
	for (int k = 0; k < W; ++k)
		atomicAdd(grad + O::W2 + W * i + k, gW2[k]);
	atomicAdd(grad + O::B2 + i, gb2);
	atomicAdd(grad + O::W3 + i, gW3);
	if (i == 0)
	{
		atomicAdd(grad + O::B3, gb3);
		atomicAdd(loss, lsum);
	}
}

__global__ void k_adam(int n, float *__restrict__ p, float const *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		float gi = g[i];
		float mi = b1 * m[i] + (1.f - b1) * gi;
		float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

template <class F> int mlp_api(F &&f) { return api_call(f); }

struct DevBuf
{
	void *p = nullptr;
	explicit DevBuf(size_t bytes)
	{
		if (bytes)
			MESH_CUDA(cudaMalloc(&p, bytes));
	}
	~DevBuf() { cudaFree(p); }
	template <class T> T *as() { return static_cast<T *>(p); }
};

template <int W> void launch_grad(cudaStream_t s, int nb, int const *idx, float const *x, float const *t,
                                  float const *params, float inv_n, float *grad, double *loss, int num_sms)
{
	int chunk = std::max(16, (nb + num_sms * 8 - 1) / (num_sms * 8));
	int blocks = (nb + chunk - 1) / chunk;
	k_mlp_grad<W><<<blocks, W, 0, s>>>(nb, idx, x, t, params, chunk, inv_n, grad, loss);
	MESH_LAUNCH_CHECK();
}

void check_width(int w) { require(w == 32 || w == 64, "MLP width must be 32 or 64"); }

} // namespace

// device-side inference for callers inside the library (the learned
// multiplier table of Fourier-accelerated gauge fixing)
void meshgb::mlp_forward_device(Context &c, int n, float const *d_x, float const *d_params, int width, bool bf16,
                                float *d_y)
{
	check_width(width);
	if (n <= 0)
		return;
	unsigned blocks = unsigned(std::max(1, std::min((n + 127) / 128, c.num_sms * 8)));
	size_t sm = sizeof(float) * size_t(nparams(width));
	if (width == 64)
	{
		if (bf16)
			k_mlp_forward<64, true><<<blocks, 128, sm, c.stream>>>(n, d_x, d_params, d_y);
		else
			k_mlp_forward<64, false><<<blocks, 128, sm, c.stream>>>(n, d_x, d_params, d_y);
	}
	else
	{
		if (bf16)
			k_mlp_forward<32, true><<<blocks, 128, sm, c.stream>>>(n, d_x, d_params, d_y);
		else
			k_mlp_forward<32, false><<<blocks, 128, sm, c.stream>>>(n, d_x, d_params, d_y);
	}
	MESH_LAUNCH_CHECK();
}

extern "C" {

int mesh_mlp_nparams(int width) { return nparams(width); }

// y[n] = MLP(x[n][3]); host arrays; bf16 != 0: BF16 inference
int mesh_mlp_forward(mesh_ctx ctx_handle, int n, float const *x, float const *params, int width, int bf16, float *y)
{
	return mlp_api([&] {
		require(ctx_handle != nullptr && x && params && y && n >= 0, "invalid argument");
		check_width(width);
		Context &c = ctx_handle->c;
		DeviceGuard dg(c.device);
		int np = nparams(width);
		DevBuf dx(sizeof(float) * 3 * size_t(n) + 16), dp(sizeof(float) * size_t(np)), dy(sizeof(float) * size_t(n) + 16);
		MESH_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemcpyAsync(dp.p, params, sizeof(float) * size_t(np), cudaMemcpyHostToDevice, c.stream));
		unsigned blocks = unsigned(std::max(1, std::min((n + 127) / 128, c.num_sms * 8)));
		size_t sm = sizeof(float) * size_t(np);
		if (n > 0)
		{
			if (width == 64)
			{
				if (bf16)
					k_mlp_forward<64, true><<<blocks, 128, sm, c.stream>>>(n, dx.as<float>(), dp.as<float>(), dy.as<float>());
				else
					k_mlp_forward<64, false><<<blocks, 128, sm, c.stream>>>(n, dx.as<float>(), dp.as<float>(), dy.as<float>());
			}
			else
			{
				if (bf16)
					k_mlp_forward<32, true><<<blocks, 128, sm, c.stream>>>(n, dx.as<float>(), dp.as<float>(), dy.as<float>());
				else
					k_mlp_forward<32, false><<<blocks, 128, sm, c.stream>>>(n, dx.as<float>(), dp.as<float>(), dy.as<float>());
			}
			MESH_LAUNCH_CHECK();
		}
		MESH_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(float) * size_t(n), cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaStreamSynchronize(c.stream));
	});
}

// full-batch mean-squared-error loss and its gradient (host arrays)
int mesh_mlp_grad(mesh_ctx ctx_handle, int n, float const *x, float const *t, float const *params, int width,
                  double *loss, float *grad)
{
	return mlp_api([&] {
		require(ctx_handle != nullptr && x && t && params && grad && n > 0, "invalid argument");
		check_width(width);
		Context &c = ctx_handle->c;
		DeviceGuard dg(c.device);
		int np = nparams(width);
		DevBuf dx(sizeof(float) * 3 * size_t(n)), dt(sizeof(float) * size_t(n)), dp(sizeof(float) * size_t(np)),
		    dg_(sizeof(float) * size_t(np)), dl(sizeof(double));
		MESH_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemcpyAsync(dt.p, t, sizeof(float) * size_t(n), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemcpyAsync(dp.p, params, sizeof(float) * size_t(np), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemsetAsync(dg_.p, 0, sizeof(float) * size_t(np), c.stream));
		MESH_CUDA(cudaMemsetAsync(dl.p, 0, sizeof(double), c.stream));
		if (width == 64)
			launch_grad<64>(c.stream, n, nullptr, dx.as<float>(), dt.as<float>(), dp.as<float>(), 1.f / float(n),
			                dg_.as<float>(), dl.as<double>(), c.num_sms);
		else
			launch_grad<32>(c.stream, n, nullptr, dx.as<float>(), dt.as<float>(), dp.as<float>(), 1.f / float(n),
			                dg_.as<float>(), dl.as<double>(), c.num_sms);
		double l = 0;
		MESH_CUDA(cudaMemcpyAsync(grad, dg_.p, sizeof(float) * size_t(np), cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaMemcpyAsync(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaStreamSynchronize(c.stream));
		if (loss)
			*loss = l / double(n);
	});
}

// Adam training on the device: `epochs` passes over the n samples in
// shuffled minibatches; params updated in place; loss_per_epoch (may be NULL)
// receives the mean training loss of each epoch.
int mesh_mlp_train(mesh_ctx ctx_handle, int n, float const *x, float const *t, float *params, int width, int epochs,
                   int batch, float lr, uint64_t seed, float *loss_per_epoch)
{
	return mlp_api([&] {
		require(ctx_handle != nullptr && x && t && params && n > 0 && epochs >= 0 && batch >= 1 && lr > 0,
		        "invalid argument");
		check_width(width);
		Context &c = ctx_handle->c;
		DeviceGuard dg(c.device);
		int np = nparams(width);
		DevBuf dx(sizeof(float) * 3 * size_t(n)), dt(sizeof(float) * size_t(n)), dp(sizeof(float) * size_t(np)),
		    dgr(sizeof(float) * size_t(np)), dm(sizeof(float) * size_t(np)), dv(sizeof(float) * size_t(np)),
		    didx(sizeof(int) * size_t(n)), dl(sizeof(double));
		MESH_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemcpyAsync(dt.p, t, sizeof(float) * size_t(n), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemcpyAsync(dp.p, params, sizeof(float) * size_t(np), cudaMemcpyHostToDevice, c.stream));
		MESH_CUDA(cudaMemsetAsync(dm.p, 0, sizeof(float) * size_t(np), c.stream));
		MESH_CUDA(cudaMemsetAsync(dv.p, 0, sizeof(float) * size_t(np), c.stream));
		std::vector<int> perm(static_cast<size_t>(n));
		std::iota(perm.begin(), perm.end(), 0);
		std::mt19937_64 rng(seed);
		int step = 0;
		const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
		for (int e = 0; e < epochs; ++e)
		{
			std::shuffle(perm.begin(), perm.end(), rng);
			MESH_CUDA(cudaMemcpyAsync(didx.p, perm.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, c.stream));
			MESH_CUDA(cudaMemsetAsync(dl.p, 0, sizeof(double), c.stream));
			for (int b0 = 0; b0 < n; b0 += batch)
			{
				int nb = std::min(batch, n - b0);
				MESH_CUDA(cudaMemsetAsync(dgr.p, 0, sizeof(float) * size_t(np), c.stream));
				if (width == 64)
					launch_grad<64>(c.stream, nb, didx.as<int>() + b0, dx.as<float>(), dt.as<float>(), dp.as<float>(),
					                1.f / float(nb), dgr.as<float>(), dl.as<double>(), c.num_sms);
				else
					launch_grad<32>(c.stream, nb, didx.as<int>() + b0, dx.as<float>(), dt.as<float>(), dp.as<float>(),
					                1.f / float(nb), dgr.as<float>(), dl.as<double>(), c.num_sms);
				++step;
				float c1 = 1.f - std::pow(b1, float(step)), c2 = 1.f - std::pow(b2, float(step));
				k_adam<<<(np + 255) / 256, 256, 0, c.stream>>>(np, dp.as<float>(), dgr.as<float>(), dm.as<float>(),
				                                               dv.as<float>(), lr, b1, b2, eps, c1, c2);
				MESH_LAUNCH_CHECK();
			}
			if (loss_per_epoch)
			{
				double l = 0;
				MESH_CUDA(cudaMemcpyAsync(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
				MESH_CUDA(cudaStreamSynchronize(c.stream));
				loss_per_epoch[e] = float(l / double(n));
			}
		}
		MESH_CUDA(cudaMemcpyAsync(params, dp.p, sizeof(float) * size_t(np), cudaMemcpyDeviceToHost, c.stream));
		MESH_CUDA(cudaStreamSynchronize(c.stream));
	});
}

} // extern "C"
