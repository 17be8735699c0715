// Learned element-block preconditioner: a per-element MLP with the library's own training and inference kernels.
//
// Input  x_e = [ u_e (the element's n_s*n_var solution coefficients), log10(dtau) ]           (d_in = nb + 1)
// Output P_e = I + reshape(W3 relu(W2 relu(W1 x_e + b1) + b2) + b3)  ~  (1/dtau + rho) (I/dtau - dF/du)_ee^-1
// i.e. the network predicts the block inverse of the pseudo-transient Newton matrix normalised by 1/dtau + rho,
// rho the mean inf-norm of the element blocks of dF/du seen in training (identity for small dtau, an O(1) matrix
// for large dtau).  Training pairs come from the block-Jacobi solve: after each assembly the exact inverses are
// formed from the batched LU factors and stored with their inputs (mlp_collect).  Loss: mean squared error over
// the nb*nb entries; optimiser: Adam.  The GEMMs are FP32 tiled kernels written here (no cuBLAS).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "dpg_gpu_internal.cuh"
#include "tc_sm100.cuh"

namespace dpg {

// ------------------------------------------------------------------------------------------------------------
// GEMM on the 5th-generation tensor cores: C[M x N] = alpha * op(A) * op(B) + beta * C, all row-major FP32 in global
// memory; op(A) is M x K, op(B) is K x N.  Each operand is rounded to BF16 (round to nearest even) as it is staged
// into shared memory and the products accumulate in FP32 in tensor memory: kind::f16 tcgen05.mma with BF16 inputs.
//
// One CTA of 128 threads computes a 128 x 128 tile of C.  K advances in chunks of 64: all threads load the A and B
// chunk from global memory (reading along whichever index is contiguous, so the transposed forms stay coalesced),
// convert to BF16 pairs and store them K-major (core matrices of 8 rows x 16 bytes, tc_sm100.cuh) into one of two
// shared-memory stages; warp 0 then issues the chunk's 4 MMAs (K = 16 each) from one elected lane and commits them to
// the stage's mbarrier, which the loaders wait on before they overwrite that stage two chunks later.  The 128 x 128
// FP32 accumulator occupies 128 TMEM columns; the epilogue reads each warp's 32 lanes (rows) with tcgen05.ld.
// Every mbarrier wait is bounded: a wait that gives up sets *err, the kernel still waits (bounded) for its own MMAs
// and frees its TMEM.
// ------------------------------------------------------------------------------------------------------------
constexpr int kGemmBM = 128, kGemmBN = 128, kGemmBK = 64;
constexpr uint32_t kGemmStageBytes = (kGemmBM + kGemmBN) * kGemmBK * 2;   // A and B chunk, BF16
constexpr size_t kGemmSmem = 2 * kGemmStageBytes + 1024;

// Stage a rows x 64 chunk of op(X) (row r, k) into K-major BF16 core matrices.  xt: op(X)[r][k] = X[k * ld + r].
// 128 threads, 32 element pairs each; the global loads of 8 pairs are issued before any of them is converted and
// stored, so a thread has 16 loads in flight instead of one dependent chain per pair.
constexpr int kGemmThreads = 128;
constexpr int kGemmPairs = kGemmBM * kGemmBK / 2 / kGemmThreads;   // 32
constexpr int kGemmBatch = 8;
__device__ __forceinline__ void gemm_stage(uint8_t* dst, const float* __restrict__ X, int ld, bool xt, int r0, int rmax,
                                           int k0, int kmax)
{
#pragma unroll
	for (int g = 0; g < kGemmPairs; g += kGemmBatch) {
		float v0[kGemmBatch], v1[kGemmBatch];
		int rr[kGemmBatch], kk[kGemmBatch];
#pragma unroll
		for (int u = 0; u < kGemmBatch; ++u) {
			const int i = threadIdx.x + (g + u) * kGemmThreads;
			int r, kp;
			if (xt) { kp = i / kGemmBM; r = i - kp * kGemmBM; }   // consecutive threads along r (contiguous in memory)
			else    { r = i / (kGemmBK / 2); kp = i - r * (kGemmBK / 2); }   // consecutive threads along k
			rr[u] = r; kk[u] = kp;
			const int gr = r0 + r, gk = k0 + 2 * kp;
			v0[u] = 0.f; v1[u] = 0.f;
			if (gr < rmax) {
				if (xt) {
					if (gk < kmax) v0[u] = X[(size_t)gk * ld + gr];
					if (gk + 1 < kmax) v1[u] = X[(size_t)(gk + 1) * ld + gr];
				} else {
					if (gk < kmax) v0[u] = X[(size_t)gr * ld + gk];
					if (gk + 1 < kmax) v1[u] = X[(size_t)gr * ld + gk + 1];
				}
			}
		}
#pragma unroll
		for (int u = 0; u < kGemmBatch; ++u) {
			const __nv_bfloat162 b = __floats2bfloat162_rn(v0[u], v1[u]);   // low half: element k
			*reinterpret_cast<__nv_bfloat162*>(dst + tc::kmajor_offset(rr[u], 2 * kk[u], kGemmBK, 2)) = b;
		}
	}
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_tc(int M, int N, int K, float alpha, const float* __restrict__ A, int lda,
                                                 const float* __restrict__ B, int ldb, float beta, float* __restrict__ C,
                                                 int ldc, int* __restrict__ err, long long polls)
{
	extern __shared__ __align__(1024) uint8_t gsm[];
	uint8_t* base = gsm + ((1024 - (tc::smem_u32(gsm) & 1023)) & 1023);
	__shared__ uint64_t bar[2];
	__shared__ uint32_t tmem_base;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int m0 = blockIdx.y * kGemmBM, n0 = blockIdx.x * kGemmBN;
	if (warp == 0) tc::tmem_alloc(&tmem_base, kGemmBN);
	if (threadIdx.x == 0) { tc::mbar_init(&bar[0], 1); tc::mbar_init(&bar[1], 1); tc::fence_mbar_init(); }
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = tmem_base;
	const int nk = (K + kGemmBK - 1) / kGemmBK;
	constexpr uint32_t idesc = tc::make_idesc(kGemmBM, kGemmBN, 1);
	// every decision to give up is made for the whole block (__syncthreads_or), so no barrier is left half-reached;
	// n_issued counts the chunks whose MMAs were issued and committed
	bool fail = false;
	int n_issued = 0;
	for (int kt = 0; kt < nk; ++kt) {
		const int st = kt & 1;
		if (kt >= 2) {
			const bool f = !tc::mbar_wait(&bar[st], (uint32_t)((kt / 2 - 1) & 1), polls);
			if (__syncthreads_or(f)) { fail = true; break; }
		}
		uint8_t* sA = base + st * kGemmStageBytes;
		uint8_t* sB = sA + kGemmBM * kGemmBK * 2;
		gemm_stage(sA, A, lda, TA, m0, M, kt * kGemmBK, K);
		gemm_stage(sB, B, ldb, !TB, n0, N, kt * kGemmBK, K);   // B staged as op(B)^T: N rows of K
		tc::fence_async_smem();
		tc::fence_before_sync();
		__syncthreads();
		if (warp == 0) {
			tc::fence_after_sync();
			const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll
			for (int kk = 0; kk < kGemmBK / 16; ++kk) {
				const uint64_t ad = tc::make_sdesc(a0 + 256 * kk, 128, (kGemmBK * 2 / 16) * 128);
				const uint64_t bd = tc::make_sdesc(b0 + 256 * kk, 128, (kGemmBK * 2 / 16) * 128);
				tc::mma_bf16_elect(tmem, ad, bd, idesc, (kt > 0 || kk > 0) ? 1u : 0u);
			}
			tc::mma_commit_elect(&bar[st]);
		}
		n_issued = kt + 1;
	}
	// every issued MMA of the tile: the last issued chunk's commit (commits track all earlier MMAs of the thread)
	const int last = n_issued - 1;
	if (!fail) fail = __syncthreads_or(!tc::mbar_wait(&bar[last & 1], (uint32_t)((last / 2) & 1), polls));
	if (fail) {
		// report, then let the issued MMAs finish before the accumulator's TMEM is released (MMAs always complete:
		// this drain has the long limit whatever the caller's one)
		const bool drained = tc::mbar_wait(&bar[last & 1], (uint32_t)((last / 2) & 1), 1ll << 24);
		if (threadIdx.x == 0) atomicExch(err, drained ? 1 : 2);
	}
	tc::fence_after_sync();
	if (!fail) {
		const int row = m0 + warp * 32 + lane;
		const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
		for (int c0 = 0; c0 < kGemmBN; c0 += 8) {
			float v[8];
			tc::tmem_ld8(taddr + c0, v);
			tc::tmem_ld_wait();
			if (row < M)
#pragma unroll
				for (int j = 0; j < 8; ++j) {
					const int col = n0 + c0 + j;
					if (col < N) {
						float* cp = C + (size_t)row * ldc + col;
						*cp = alpha * v[j] + (beta == 0.f ? 0.f : beta * *cp);
					}
				}
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) { tc::tmem_relinquish(); tc::tmem_dealloc(tmem, kGemmBN); }
}

static int* g_gemm_err = nullptr;   // error flag of the bounded waits (device), allocated with the first MLP
constexpr long long kGemmPolls = 1ll << 22;   // poll limit of a bounded wait (far beyond any MMA's latency)
static long long g_gemm_polls = kGemmPolls;   // changed only by the test hook dpg_gpu_mlp_set_wait_limit

static void gemm(cudaStream_t s, bool ta, bool tb, int M, int N, int K, float alpha, const float* A, int lda,
                 const float* B, int ldb, float beta, float* C, int ldc)
{
	dim3 grid((N + kGemmBN - 1) / kGemmBN, (M + kGemmBM - 1) / kGemmBM);
	const long long p = g_gemm_polls;
	if (!ta && !tb) k_gemm_tc<false, false><<<grid, 128, kGemmSmem, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, g_gemm_err, p);
	else if (!ta && tb) k_gemm_tc<false, true><<<grid, 128, kGemmSmem, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, g_gemm_err, p);
	else if (ta && !tb) k_gemm_tc<true, false><<<grid, 128, kGemmSmem, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, g_gemm_err, p);
	else k_gemm_tc<true, true><<<grid, 128, kGemmSmem, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, g_gemm_err, p);
}

static int gemm_setup()
{
	if (!g_gemm_err) {
		if (cudaMalloc(&g_gemm_err, sizeof(int)) != cudaSuccess) return DPG_ERR_CUDA;
		if (cudaMemset(g_gemm_err, 0, sizeof(int)) != cudaSuccess) return DPG_ERR_CUDA;
	}
	cudaError_t e = cudaSuccess;
	e = cudaFuncSetAttribute(k_gemm_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem); if (e) return DPG_ERR_CUDA;
	e = cudaFuncSetAttribute(k_gemm_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem); if (e) return DPG_ERR_CUDA;
	e = cudaFuncSetAttribute(k_gemm_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem); if (e) return DPG_ERR_CUDA;
	e = cudaFuncSetAttribute(k_gemm_tc<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem); if (e) return DPG_ERR_CUDA;
	return DPG_OK;
}

// non-zero if a bounded wait of a GEMM gave up since the last call (cleared)
static int gemm_error(cudaStream_t s)
{
	int h = 0;
	if (!g_gemm_err) return 0;
	if (cudaMemcpyAsync(&h, g_gemm_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
	if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
	if (h) cudaMemsetAsync(g_gemm_err, 0, sizeof(int), s);
	return h;
}

__global__ void k_bias_act(int rows, int cols, const float* __restrict__ b, float* __restrict__ Y, int relu)
{
	const int64_t n = (int64_t)rows * cols;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		float v = Y[i] + b[i % cols];
		Y[i] = relu ? fmaxf(v, 0.f) : v;
	}
}

__global__ void k_relu_mask(int64_t n, const float* __restrict__ act, float* __restrict__ g)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		if (act[i] <= 0.f) g[i] = 0.f;
}

// db[j] = sum_r G[r][j]
__global__ void k_colsum(int rows, int cols, const float* __restrict__ G, float* __restrict__ db)
{
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= cols) return;
	float s = 0.f;
	for (int r = 0; r < rows; ++r) s += G[(size_t)r * cols + j];
	db[j] = s;
}

// out = net output (without the identity); G = 2/(batch*d_out) * (I + out - T); loss partial sums per block
__global__ void k_mse(int batch, int nb, const float* __restrict__ out, const float* __restrict__ T,
                      float* __restrict__ G, double* __restrict__ loss_part)
{
	__shared__ double red[8];
	const int64_t n = (int64_t)batch * nb * nb;
	const double scale = 2.0 / (double)n;
	double acc = 0.0;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int64_t w = i % ((int64_t)nb * nb);
		const float id = ((w / nb) == (w % nb)) ? 1.f : 0.f;
		const float d = id + out[i] - T[i];
		acc += (double)d * d;
		G[i] = (float)(scale * d);
	}
	for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int i = 0; i < (int)(blockDim.x / 32); ++i) t += red[i];
		loss_part[blockIdx.x] = t;
	}
}

__global__ void k_adam(int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float c1, float c2)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		m1[i] = b1 * m1[i] + (1.f - b1) * gi;
		m2[i] = b2 * m2[i] + (1.f - b2) * gi * gi;
		w[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + 1e-8f);
	}
}

// features of every element: [u_e, log10(dtau_e)] (FP32), shift_e = 1/dtau_e
__global__ void k_features(int n_vol, int nb, const double* __restrict__ u, const double* __restrict__ shift,
                           float* __restrict__ X)
{
	const int d_in = nb + 1;
	const int64_t n = (int64_t)n_vol * d_in;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int e = (int)(i / d_in), k = (int)(i - (int64_t)e * d_in);
		X[i] = (k < nb) ? (float)u[(int64_t)e * nb + k] : (float)(-log10(shift[e]));
	}
}

// T_e = (shift_e + rho) (LU_e)^-1 (shift_e = 1/dtau_e), one thread block per element: columns solved in parallel
__global__ void k_lu_inverse_scaled(int nb, const double* __restrict__ lu, const int* __restrict__ piv,
                                    const double* __restrict__ shift, double rho, float* __restrict__ T)
{
	extern __shared__ double sh[];
	double* a = sh;                 // nb x nb
	const int e = blockIdx.x;
	const double scale = shift[e] + rho;
	for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) a[i] = lu[(int64_t)e * nb * nb + i];
	__syncthreads();
	for (int col = threadIdx.x; col < nb; col += blockDim.x) {
		double x[128];
		for (int i = 0; i < nb; ++i) x[i] = (i == col) ? 1.0 : 0.0;
		for (int k = 0; k < nb; ++k) {
			const int p = piv[(int64_t)e * nb + k];
			if (p != k) { const double t = x[k]; x[k] = x[p]; x[p] = t; }
		}
		for (int i = 0; i < nb; ++i) {
			double s = x[i];
			for (int j = 0; j < i; ++j) s -= a[i * nb + j] * x[j];
			x[i] = s;
		}
		for (int i = nb - 1; i >= 0; --i) {
			double s = x[i];
			for (int j = i + 1; j < nb; ++j) s -= a[i * nb + j] * x[j];
			x[i] = s / a[i * nb + i];
		}
		for (int i = 0; i < nb; ++i) T[((int64_t)e * nb + i) * nb + col] = (float)(scale * x[i]);
	}
}

__global__ void k_add_identity(int n_vol, int nb, float* __restrict__ P)
{
	const int64_t n = (int64_t)n_vol * nb;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int e = (int)(i / nb), k = (int)(i - (int64_t)e * nb);
		P[((int64_t)e * nb + k) * nb + k] += 1.f;
	}
}

// ------------------------------------------------------------------------------------------------------------
struct Mlp {
	int nb = 0, d_in = 0, hid = 0, d_out = 0;
	int cap = 0, n_samples = 0, n_vol = 0;
	float* params = nullptr;   // W1 [hid x d_in], b1, W2 [hid x hid], b2, W3 [d_out x hid], b3
	float* grads = nullptr;
	float *m1 = nullptr, *m2 = nullptr;
	int64_t n_params = 0;
	int64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
	float* sX = nullptr;       // samples [cap][d_in]
	float* sT = nullptr;       // samples [cap][d_out]
	float *X = nullptr, *H1 = nullptr, *H2 = nullptr, *Y = nullptr, *G = nullptr, *G1 = nullptr, *G2 = nullptr;
	int buf_rows = 0;
	float* P = nullptr;        // predictions for all elements [n_vol][d_out]
	float* feat = nullptr;     // [n_vol][d_in]
	double* loss_part = nullptr;
	int adam_t = 0;
	double rho = 0.0;          // running mean of the block norms of the collected samples
	int rho_count = 0;
};

static int grid1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

void mlp_free(dpg_gpu_ctx* c)
{
	Mlp* m = (Mlp*)c->mlp;
	if (!m) return;
	void* ptrs[] = {m->params, m->grads, m->m1, m->m2, m->sX, m->sT, m->X, m->H1, m->H2, m->Y, m->G, m->G1, m->G2, m->P,
	                m->feat, m->loss_part};
	for (void* p : ptrs) if (p) cudaFree(p);
	delete m;
	c->mlp = nullptr;
}

static int ensure_rows(Mlp* m, int rows)
{
	if (rows <= m->buf_rows) return DPG_OK;
	void* ptrs[] = {m->X, m->H1, m->H2, m->Y, m->G, m->G1, m->G2};
	for (void* p : ptrs) if (p) cudaFree(p);
	bool ok = cudaMalloc(&m->X, sizeof(float) * (size_t)rows * m->d_in) == cudaSuccess;
	ok = ok && cudaMalloc(&m->H1, sizeof(float) * (size_t)rows * m->hid) == cudaSuccess;
	ok = ok && cudaMalloc(&m->H2, sizeof(float) * (size_t)rows * m->hid) == cudaSuccess;
	ok = ok && cudaMalloc(&m->Y, sizeof(float) * (size_t)rows * m->d_out) == cudaSuccess;
	ok = ok && cudaMalloc(&m->G, sizeof(float) * (size_t)rows * m->d_out) == cudaSuccess;
	ok = ok && cudaMalloc(&m->G1, sizeof(float) * (size_t)rows * m->hid) == cudaSuccess;
	ok = ok && cudaMalloc(&m->G2, sizeof(float) * (size_t)rows * m->hid) == cudaSuccess;
	m->buf_rows = ok ? rows : 0;
	return ok ? DPG_OK : DPG_ERR_CUDA;
}

// forward for `rows` inputs in X -> H1, H2, Y (Y without the identity)
static void forward(cudaStream_t s, Mlp* m, const float* X, int rows, float* H1, float* H2, float* Y)
{
	const float* W = m->params;
	gemm(s, false, true, rows, m->hid, m->d_in, 1.f, X, m->d_in, W + m->oW1, m->d_in, 0.f, H1, m->hid);
	k_bias_act<<<grid1((int64_t)rows * m->hid), 256, 0, s>>>(rows, m->hid, W + m->ob1, H1, 1);
	gemm(s, false, true, rows, m->hid, m->hid, 1.f, H1, m->hid, W + m->oW2, m->hid, 0.f, H2, m->hid);
	k_bias_act<<<grid1((int64_t)rows * m->hid), 256, 0, s>>>(rows, m->hid, W + m->ob2, H2, 1);
	gemm(s, false, true, rows, m->d_out, m->hid, 1.f, H2, m->hid, W + m->oW3, m->hid, 0.f, Y, m->d_out);
	k_bias_act<<<grid1((int64_t)rows * m->d_out), 256, 0, s>>>(rows, m->d_out, W + m->ob3, Y, 0);
}

// loss and parameter gradient (into m->grads) of one batch already in m->X / target T
static int loss_grad(cudaStream_t s, Mlp* m, int rows, const float* X, const float* T, double* loss)
{
	forward(s, m, X, rows, m->H1, m->H2, m->Y);
	const int nblk = 256;
	k_mse<<<nblk, 256, 0, s>>>(rows, m->nb, m->Y, T, m->G, m->loss_part);
	float* g = m->grads;
	const float* W = m->params;
	// layer 3
	gemm(s, true, false, m->d_out, m->hid, rows, 1.f, m->G, m->d_out, m->H2, m->hid, 0.f, g + m->oW3, m->hid);
	k_colsum<<<(m->d_out + 255) / 256, 256, 0, s>>>(rows, m->d_out, m->G, g + m->ob3);
	gemm(s, false, false, rows, m->hid, m->d_out, 1.f, m->G, m->d_out, W + m->oW3, m->hid, 0.f, m->G2, m->hid);
	k_relu_mask<<<grid1((int64_t)rows * m->hid), 256, 0, s>>>((int64_t)rows * m->hid, m->H2, m->G2);
	// layer 2
	gemm(s, true, false, m->hid, m->hid, rows, 1.f, m->G2, m->hid, m->H1, m->hid, 0.f, g + m->oW2, m->hid);
	k_colsum<<<(m->hid + 255) / 256, 256, 0, s>>>(rows, m->hid, m->G2, g + m->ob2);
	gemm(s, false, false, rows, m->hid, m->hid, 1.f, m->G2, m->hid, W + m->oW2, m->hid, 0.f, m->G1, m->hid);
	k_relu_mask<<<grid1((int64_t)rows * m->hid), 256, 0, s>>>((int64_t)rows * m->hid, m->H1, m->G1);
	// layer 1
	gemm(s, true, false, m->hid, m->d_in, rows, 1.f, m->G1, m->hid, X, m->d_in, 0.f, g + m->oW1, m->d_in);
	k_colsum<<<(m->hid + 255) / 256, 256, 0, s>>>(rows, m->hid, m->G1, g + m->ob1);
	if (loss) {
		std::vector<double> parts(nblk);
		if (cudaMemcpyAsync(parts.data(), m->loss_part, 8 * nblk, cudaMemcpyDeviceToHost, s) != cudaSuccess) return DPG_ERR_CUDA;
		if (cudaStreamSynchronize(s) != cudaSuccess) return DPG_ERR_CUDA;
		double t = 0.0;
		for (double p : parts) t += p;
		*loss = t / ((double)rows * m->d_out);
	}
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

double mlp_rho(dpg_gpu_ctx* c)
{
	Mlp* m = (Mlp*)c->mlp;
	return m ? m->rho : 0.0;
}

int mlp_collect(dpg_gpu_ctx* c, const double* u, const double* lu, const int* piv, const double* shift, double rho)
{
	Mlp* m = (Mlp*)c->mlp;
	if (!m) return DPG_OK;
	m->rho = (m->rho * m->rho_count + rho) / (m->rho_count + 1);
	++m->rho_count;
	const int n_vol = c->g.n_vol;
	const int take = std::min(n_vol, m->cap - m->n_samples);
	if (take <= 0) return DPG_OK;
	cudaStream_t s = c->stream;
	k_features<<<grid1((int64_t)take * m->d_in), 256, 0, s>>>(take, m->nb, u, shift,
	                                                          m->sX + (int64_t)m->n_samples * m->d_in);
	const size_t smem = (size_t)m->nb * m->nb * 8;
	if (smem > 48 * 1024) cudaFuncSetAttribute(k_lu_inverse_scaled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	// target (1/dtau + rho) B^-1
	k_lu_inverse_scaled<<<take, 64, smem, s>>>(m->nb, lu, piv, shift, rho, m->sT + (int64_t)m->n_samples * m->d_out);
	m->n_samples += take;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int mlp_predict(dpg_gpu_ctx* c, const double* u, const double* shift, float** P)
{
	Mlp* m = (Mlp*)c->mlp;
	if (!m) return DPG_ERR_INVALID;
	const int n_vol = c->g.n_vol;
	cudaStream_t s = c->stream;
	if (!m->P) {
		if (cudaMalloc(&m->P, sizeof(float) * (size_t)n_vol * m->d_out) != cudaSuccess) return DPG_ERR_CUDA;
		if (cudaMalloc(&m->feat, sizeof(float) * (size_t)n_vol * m->d_in) != cudaSuccess) return DPG_ERR_CUDA;
	}
	const int chunk = 8192;
	if (ensure_rows(m, std::min(chunk, n_vol))) return DPG_ERR_CUDA;
	k_features<<<grid1((int64_t)n_vol * m->d_in), 256, 0, s>>>(n_vol, m->nb, u, shift, m->feat);
	for (int r0 = 0; r0 < n_vol; r0 += chunk) {
		const int rows = std::min(chunk, n_vol - r0);
		forward(s, m, m->feat + (int64_t)r0 * m->d_in, rows, m->H1, m->H2, m->P + (int64_t)r0 * m->d_out);
	}
	k_add_identity<<<grid1((int64_t)n_vol * m->nb), 256, 0, s>>>(n_vol, m->nb, m->P);
	*P = m->P;
	if (cudaGetLastError() != cudaSuccess) return DPG_ERR_CUDA;
	const int ge = gemm_error(s);
	return ge ? (ge < 0 ? DPG_ERR_CUDA : DPG_ERR_TIMEOUT) : DPG_OK;
}

} // namespace dpg

using dpg::Mlp;

extern "C" int dpg_gpu_mlp_enable(dpg_gpu_ctx* c, int hidden, int capacity, uint64_t seed)
{
	if (!c || hidden < 8 || hidden > 4096 || capacity < 1) return DPG_ERR_INVALID;
	if (c->hp) return DPG_ERR_UNSUPPORTED;   // element blocks of one order
	dpg::mlp_free(c);
	Mlp* m = new Mlp();
	c->mlp = m;
	m->nb = c->g.n_s * c->n_var;
	m->d_in = m->nb + 1;
	m->hid = hidden;
	m->d_out = m->nb * m->nb;
	m->cap = capacity;
	m->n_vol = c->g.n_vol;
	m->oW1 = 0; m->ob1 = m->oW1 + (int64_t)hidden * m->d_in;
	m->oW2 = m->ob1 + hidden; m->ob2 = m->oW2 + (int64_t)hidden * hidden;
	m->oW3 = m->ob2 + hidden; m->ob3 = m->oW3 + (int64_t)m->d_out * hidden;
	m->n_params = m->ob3 + m->d_out;
	std::vector<float> w((size_t)m->n_params, 0.f);
	uint64_t st = seed * 0x9E3779B97F4A7C15ull + 12345;
	auto rnd = [&]() {
		st ^= st << 13; st ^= st >> 7; st ^= st << 17;
		return (double)(st >> 11) * (1.0 / 9007199254740992.0);
	};
	auto init = [&](int64_t off, int64_t n, double fan_in, double gain) {
		const double a = gain * std::sqrt(6.0 / fan_in);
		for (int64_t i = 0; i < n; ++i) w[(size_t)(off + i)] = (float)((2.0 * rnd() - 1.0) * a);
	};
	init(m->oW1, (int64_t)hidden * m->d_in, m->d_in, 1.0);
	init(m->oW2, (int64_t)hidden * hidden, hidden, 1.0);
	init(m->oW3, (int64_t)m->d_out * hidden, hidden, 0.01);   // start close to the identity preconditioner
	bool ok = cudaMalloc(&m->params, 4 * (size_t)m->n_params) == cudaSuccess;
	ok = ok && cudaMalloc(&m->grads, 4 * (size_t)m->n_params) == cudaSuccess;
	ok = ok && cudaMalloc(&m->m1, 4 * (size_t)m->n_params) == cudaSuccess;
	ok = ok && cudaMalloc(&m->m2, 4 * (size_t)m->n_params) == cudaSuccess;
	ok = ok && cudaMalloc(&m->sX, 4 * (size_t)capacity * m->d_in) == cudaSuccess;
	ok = ok && cudaMalloc(&m->sT, 4 * (size_t)capacity * m->d_out) == cudaSuccess;
	ok = ok && cudaMalloc(&m->loss_part, 8 * 256) == cudaSuccess;
	if (!ok || dpg::gemm_setup()) { dpg::mlp_free(c); return DPG_ERR_CUDA; }
	cudaMemcpy(m->params, w.data(), 4 * (size_t)m->n_params, cudaMemcpyHostToDevice);
	cudaMemset(m->m1, 0, 4 * (size_t)m->n_params);
	cudaMemset(m->m2, 0, 4 * (size_t)m->n_params);
	return DPG_OK;
}

extern "C" int dpg_gpu_mlp_samples(dpg_gpu_ctx* c)
{
	if (!c || !c->mlp) return 0;
	return ((Mlp*)c->mlp)->n_samples;
}

extern "C" int dpg_gpu_mlp_dims(dpg_gpu_ctx* c, int* d_in, int* hidden, int* d_out)
{
	if (!c || !c->mlp) return DPG_ERR_INVALID;
	Mlp* m = (Mlp*)c->mlp;
	if (d_in) *d_in = m->d_in;
	if (hidden) *hidden = m->hid;
	if (d_out) *d_out = m->d_out;
	return DPG_OK;
}

extern "C" int dpg_gpu_mlp_train(dpg_gpu_ctx* c, int epochs, int batch, double lr, double* loss_out)
{
	if (!c || !c->mlp || epochs < 0 || batch < 1) return DPG_ERR_INVALID;
	Mlp* m = (Mlp*)c->mlp;
	if (m->n_samples < 1) return DPG_ERR_INVALID;
	batch = std::min(batch, m->n_samples);
	if (dpg::ensure_rows(m, batch)) return DPG_ERR_CUDA;
	cudaStream_t s = c->stream;
	double last = 0.0;
	const float b1 = 0.9f, b2 = 0.999f;
	for (int ep = 0; ep < epochs; ++ep) {
		double sum = 0.0;
		int nb_done = 0;
		for (int r0 = 0; r0 + batch <= m->n_samples; r0 += batch) {
			double loss = 0.0;
			const bool want = (r0 + 2 * batch > m->n_samples);   // last batch of the epoch reports the loss
			int rc = dpg::loss_grad(s, m, batch, m->sX + (int64_t)r0 * m->d_in, m->sT + (int64_t)r0 * m->d_out,
			                        want ? &loss : nullptr);
			if (rc) return rc;
			++m->adam_t;
			const float c1 = 1.f - powf(b1, (float)m->adam_t), c2 = 1.f - powf(b2, (float)m->adam_t);
			dpg::k_adam<<<dpg::grid1(m->n_params), 256, 0, s>>>(m->n_params, m->params, m->grads, m->m1, m->m2, (float)lr,
			                                                     b1, b2, c1, c2);
			if (want) { sum += loss; ++nb_done; }
		}
		if (nb_done) last = sum / nb_done;
	}
	if (cudaStreamSynchronize(s) != cudaSuccess) return DPG_ERR_CUDA;
	const int ge = dpg::gemm_error(s);
	if (ge) return ge < 0 ? DPG_ERR_CUDA : DPG_ERR_TIMEOUT;
	if (loss_out) *loss_out = last;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

extern "C" int dpg_gpu_mlp_set_wait_limit(dpg_gpu_ctx* c, long long polls)
{
	if (!c || !c->mlp) return DPG_ERR_INVALID;
	dpg::g_gemm_polls = polls < 0 ? dpg::kGemmPolls : polls;
	return DPG_OK;
}

extern "C" int dpg_gpu_mlp_params(dpg_gpu_ctx* c, float* get, const float* set, int64_t* n)
{
	if (!c || !c->mlp) return DPG_ERR_INVALID;
	Mlp* m = (Mlp*)c->mlp;
	if (n) *n = m->n_params;
	if (set && cudaMemcpy(m->params, set, 4 * (size_t)m->n_params, cudaMemcpyHostToDevice) != cudaSuccess) return DPG_ERR_CUDA;
	if (get && cudaMemcpy(get, m->params, 4 * (size_t)m->n_params, cudaMemcpyDeviceToHost) != cudaSuccess) return DPG_ERR_CUDA;
	return DPG_OK;
}

extern "C" int dpg_gpu_mlp_loss_grad(dpg_gpu_ctx* c, int batch, const float* x, const float* target, double* loss,
                                     float* grad)
{
	if (!c || !c->mlp || batch < 1 || !x || !target) return DPG_ERR_INVALID;
	Mlp* m = (Mlp*)c->mlp;
	if (dpg::ensure_rows(m, batch)) return DPG_ERR_CUDA;
	float* dT = nullptr;
	if (cudaMalloc(&dT, 4 * (size_t)batch * m->d_out) != cudaSuccess) return DPG_ERR_CUDA;
	cudaMemcpy(m->X, x, 4 * (size_t)batch * m->d_in, cudaMemcpyHostToDevice);
	cudaMemcpy(dT, target, 4 * (size_t)batch * m->d_out, cudaMemcpyHostToDevice);
	int rc = dpg::loss_grad(c->stream, m, batch, m->X, dT, loss);
	if (!rc) { const int ge = dpg::gemm_error(c->stream); if (ge) rc = ge < 0 ? DPG_ERR_CUDA : DPG_ERR_TIMEOUT; }
	if (!rc && grad) rc = cudaMemcpy(grad, m->grads, 4 * (size_t)m->n_params, cudaMemcpyDeviceToHost) == cudaSuccess
	                           ? DPG_OK : DPG_ERR_CUDA;
	cudaFree(dT);
	return rc;
}
