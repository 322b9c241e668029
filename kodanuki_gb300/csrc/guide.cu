// The learned guide: a multiresolution hash-grid encoding of the position
// (16 levels, 2 features a level, FP16 table), a 48-64-64-64-48 ReLU network
// without biases (a constant input of 1 gives the first layer one), and its
// first 40 outputs read as eight von Mises-Fisher lobes.  Training is online
// on the radiance the tracer itself carries back to each recorded vertex,
// by the neural-importance-sampling loss mean(-w log q(direction)) and Adam.
//
// The network runs on the 5th-generation tensor cores: 128 samples a CTA,
// one a TMEM lane; each layer is tcgen05.mma (kind::f16, BF16 operands from
// shared memory in the no-swizzle K-major layout, FP32 accumulators in
// TMEM) issued by one thread and committed to an mbarrier; the epilogue
// reads its row back with tcgen05.ld, applies the ReLU and writes the next
// layer's operand.  The backward pass is two MMAs a layer: the input
// gradient (dY times W, with W's transposed image) and the weight gradient
// (dY^T times X, the batch as the contraction, M padded to 128).  The
// packed BF16 weight images come into shared memory by one bulk TMA copy.
//
// The reference has no learned guide: this is the backend's added form.
#include "guide_mix.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

struct kdn_guide {
	int device          = 0;
	int smCount         = 0;
	uint32_t tableLog2  = 19;
	float lr            = 1e-2f;
	float lo[3]         = {}, hi[3] = {};
	uint32_t step       = 0; // Adam's t
	bool ready          = false;
	float* weights      = nullptr; // FP32 master, 14336
	float* wGrad        = nullptr;
	float* wM           = nullptr;
	float* wV           = nullptr;
	float* table        = nullptr; // FP32 master, levels << log2 x 2
	float* tGrad        = nullptr;
	float* tM           = nullptr;
	float* tV           = nullptr;
	__half* tHalf       = nullptr; // what the encoding reads
	uint8_t* packed     = nullptr; // BF16 operand images of the weights and their transposes
	float* loss         = nullptr;
	uint32_t* error     = nullptr;
	float* samples      = nullptr; // gathered (or uploaded) training samples
	uint32_t* count     = nullptr;
	uint32_t capacity   = 0;
	uint32_t batch      = 16384;
	uint32_t maxSteps   = 256;
	cudaStream_t stream = nullptr;
	std::mutex lock;
};

namespace kdn {
namespace {

constexpr uint32_t kLevels = 16, kIn = 48, kHid = 64, kOutW = 48;
constexpr uint32_t kWeights = kHid * kIn + 2 * kHid * kHid + kOutW * kHid; // 14336
constexpr float kKappaLo = -2.0f, kKappaHi = 8.0f;
// operand images: W0 [64][48], W1, W2 [64][64], W3 [48][64], then the
// transposes W0t [48][64], W1t, W2t [64][64], W3t [64][48]
constexpr uint32_t kForwardImages = 28672, kPacked = 57344;
__constant__ int cRes[16] = { 16, 22, 30, 42, 58, 80, 111, 153, 212, 294, 406, 561, 776, 1072, 1482, 2048 };

__host__ __device__ constexpr uint32_t nIn(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr uint32_t nOut(int l) { return l == 3 ? kOutW : kHid; }
__host__ __device__ constexpr uint32_t wOff(int l) { return l == 0 ? 0u : l == 1 ? 3072u : l == 2 ? 7168u : 11264u; }
__host__ __device__ constexpr uint32_t imgW(int l) { return l == 0 ? 0u : l == 1 ? 6144u : l == 2 ? 14336u : 22528u; }
__host__ __device__ constexpr uint32_t imgWt(int l) { return kForwardImages + imgW(l); }

// byte offset of (r, k) in an operand image of K columns: 8x16-byte core
// matrices, K-adjacent ones 128 bytes apart, row groups of 8 K*16 apart
__host__ __device__ __forceinline__ uint32_t imgAt(uint32_t r, uint32_t k, uint32_t K) { return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u; }

// shared memory of the training kernel
constexpr uint32_t kSX0 = kPacked, kSX1 = kSX0 + 12288, kSX2 = kSX1 + 16384, kSX3 = kSX2 + 16384;
constexpr uint32_t kSDY = kSX3 + 16384, kSDYT = kSDY + 16384, kSXT = kSDYT + 32768, kSBar = kSXT + 16384;
constexpr uint32_t kTrainSmem = kSBar + 64;
// of the query kernel
constexpr uint32_t kQX0 = kForwardImages, kQXA = kQX0 + 12288, kQXB = kQXA + 16384, kQBar = kQXB + 16384;
constexpr uint32_t kQuerySmem = kQBar + 64;
constexpr uint32_t kSpin = 1u << 22; // mbarrier polls before a kernel gives up

__device__ __forceinline__ uint32_t sAddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// tcgen05 shared-memory descriptor: start >> 4, leading (K) byte offset 128,
// stride (8-row) byte offset K*16, version 1, no swizzle
__device__ __forceinline__ uint64_t descOf(uint32_t addr, uint32_t K) {
	return uint64_t((addr & 0x3FFFFu) >> 4) | (uint64_t(128u >> 4) << 16) | (uint64_t((K * 16u) >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 D, BF16 A and B, both K-major, M 128
__device__ __forceinline__ uint32_t idescOf(uint32_t N) { return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((128u >> 4) << 24); }

// D[128 x N] = A[128 x K] . B[N x K]^T, 16 of K an instruction
__device__ __forceinline__ void mma(uint32_t d, uint32_t a, uint32_t b, uint32_t K, uint32_t N) {
	const uint32_t idesc = idescOf(N);
	for (uint32_t kk = 0; kk < K / 16u; ++kk) {
		const uint64_t ad = descOf(a + kk * 256u, K);
		const uint64_t bd = descOf(b + kk * 256u, K);
		asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d), "l"(ad), "l"(bd), "r"(idesc), "r"(kk) : "memory");
	}
}
__device__ __forceinline__ void commit(uint32_t bar) { asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory"); }

__device__ __forceinline__ bool waitBar(uint32_t bar, uint32_t parity) {
	for (uint32_t i = 0; i < kSpin; ++i) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n" : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
		if (ok) return true;
	}
	return false;
}

// between stages: generic writes visible to the tensor cores, TMEM reads
// done before the next MMA
__device__ __forceinline__ void stage() {
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 columns of this thread's TMEM lane
__device__ __forceinline__ void tload16(uint32_t taddr, float* v) {
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
	    "tcgen05.wait::ld.sync.aligned;"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
	      "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr)
	    : "memory");
#pragma unroll
	for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
template <int N>
__device__ __forceinline__ void tload(uint32_t tmem, uint32_t col, float* v) {
	const uint32_t lane = (threadIdx.x >> 5) * 32u;
#pragma unroll
	for (int c = 0; c < N; c += 16) tload16(tmem + (lane << 16) + col + c, v + c);
}

template <int K>
__device__ __forceinline__ void storeRow(uint8_t* img, uint32_t r, const float* v, bool relu) {
#pragma unroll
	for (int k0 = 0; k0 < K; k0 += 8) {
		uint32_t p[4];
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			float a = v[k0 + 2 * j], b = v[k0 + 2 * j + 1];
			if (relu) {
				a = fmaxf(a, 0.0f);
				b = fmaxf(b, 0.0f);
			}
			__nv_bfloat162 h = __floats2bfloat162_rn(a, b);
			p[j]             = *reinterpret_cast<uint32_t*>(&h);
		}
		*reinterpret_cast<uint4*>(img + imgAt(r, k0, K)) = make_uint4(p[0], p[1], p[2], p[3]);
	}
}
template <int K>
__device__ __forceinline__ void readRow(const uint8_t* img, uint32_t r, float* v) {
#pragma unroll
	for (int k0 = 0; k0 < K; k0 += 8) {
		const uint4 q      = *reinterpret_cast<const uint4*>(img + imgAt(r, k0, K));
		const uint32_t p[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			__nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&p[j]);
			v[k0 + 2 * j]     = __bfloat162float(h.x);
			v[k0 + 2 * j + 1] = __bfloat162float(h.y);
		}
	}
}
// column c of a transposed image [F][128]: row f gets v[f]
template <int F>
__device__ __forceinline__ void storeColumn(uint8_t* img, uint32_t c, const float* v) {
#pragma unroll
	for (int f = 0; f < F; ++f) *reinterpret_cast<__nv_bfloat16*>(img + imgAt(f, c, 128)) = __float2bfloat16_rn(v[f]);
}

struct Region {
	float lo[3], hi[3];
};

// the 8 corners of a level's cell and their trilinear weights
__device__ __forceinline__ void cornersAt(const float u[3], int level, uint32_t tableLog2, uint32_t idx[8], float w[8]) {
	const int N     = cRes[level];
	const float fN  = float(N);
	const uint32_t T = 1u << tableLog2;
	int c0[3];
	float f[3];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const float x = u[a] * fN;
		c0[a]         = min(int(floorf(x)), N - 1);
		f[a]          = x - float(c0[a]);
	}
	const uint64_t side = uint64_t(N + 1);
	const bool dense    = side * side * side <= uint64_t(T);
#pragma unroll
	for (int c = 0; c < 8; ++c) {
		const uint32_t g0 = uint32_t(c0[0] + (c & 1)), g1 = uint32_t(c0[1] + ((c >> 1) & 1)), g2 = uint32_t(c0[2] + ((c >> 2) & 1));
		idx[c]            = dense ? g0 + uint32_t(N + 1) * (g1 + uint32_t(N + 1) * g2) : ((g0 * 1u) ^ (g1 * 2654435761u) ^ (g2 * 805459861u)) & (T - 1u);
		float wc          = 1.0f;
		wc                = __fmul_rn(wc, (c & 1) ? f[0] : 1.0f - f[0]);
		wc                = __fmul_rn(wc, ((c >> 1) & 1) ? f[1] : 1.0f - f[1]);
		wc                = __fmul_rn(wc, ((c >> 2) & 1) ? f[2] : 1.0f - f[2]);
		w[c]              = wc;
	}
}

__device__ __forceinline__ void unitOf(const Region& R, float3 p, float u[3]) {
	const float pv[3] = { p.x, p.y, p.z };
#pragma unroll
	for (int a = 0; a < 3; ++a) u[a] = fminf(fmaxf(__fdiv_rn(pv[a] - R.lo[a], R.hi[a] - R.lo[a]), 0.0f), 1.0f);
}

// the network's input: 32 grid features, the normal, 1, zeros
__device__ __forceinline__ void encodeRow(const __half2* table, uint32_t tableLog2, const Region& R, float3 p, float3 n, float x[kIn]) {
	float u[3];
	unitOf(R, p, u);
	for (int l = 0; l < int(kLevels); ++l) {
		uint32_t idx[8];
		float w[8];
		cornersAt(u, l, tableLog2, idx, w);
		const __half2* level = table + (size_t(l) << tableLog2);
		float a = 0.0f, b = 0.0f;
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			const float2 v = __half22float2(__ldg(level + idx[c]));
			a              = __fadd_rn(a, __fmul_rn(w[c], v.x));
			b              = __fadd_rn(b, __fmul_rn(w[c], v.y));
		}
		x[2 * l]     = a;
		x[2 * l + 1] = b;
	}
	x[32] = n.x;
	x[33] = n.y;
	x[34] = n.z;
	x[35] = 1.0f;
#pragma unroll
	for (int k = 36; k < int(kIn); ++k) x[k] = 0.0f;
}

// the outputs as lobes: softmax weights, clamped exp concentration, unit mean
__device__ __forceinline__ void lobesOf(const float* o, float* L) {
	float amax = o[0];
#pragma unroll
	for (int j = 1; j < kGuideLobes; ++j) amax = fmaxf(amax, o[5 * j]);
	float e[kGuideLobes], sum = 0.0f;
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		e[j] = expf(o[5 * j] - amax);
		sum += e[j];
	}
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		const float* m  = o + 5 * j + 2;
		const float nrm = sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
		const bool flat = !(nrm > 1e-6f); // read as +z
		L[5 * j]        = e[j] / sum;
		L[5 * j + 1]    = expf(fminf(fmaxf(o[5 * j + 1], kKappaLo), kKappaHi));
		L[5 * j + 2]    = flat ? 0.0f : m[0] / nrm;
		L[5 * j + 3]    = flat ? 0.0f : m[1] / nrm;
		L[5 * j + 4]    = flat ? 1.0f : m[2] / nrm;
	}
}

// mean(-w log q(d)) over the batch: this row's share and its gradient
__device__ void lossRow(const float* o, float3 d, float w, float invN, float* g, float& loss) {
	float amax = o[0];
#pragma unroll
	for (int j = 1; j < kGuideLobes; ++j) amax = fmaxf(amax, o[5 * j]);
	float pi[kGuideLobes], kap[kGuideLobes], mu[kGuideLobes][3], nrm[kGuideLobes], cs[kGuideLobes], pv[kGuideLobes];
	bool live[kGuideLobes];
	float sum = 0.0f;
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		pi[j] = expf(o[5 * j] - amax);
		sum += pi[j];
	}
	float q = 0.0f;
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		pi[j]         = pi[j] / sum;
		const float c = o[5 * j + 1];
		live[j]       = c > kKappaLo && c < kKappaHi;
		kap[j]        = expf(fminf(fmaxf(c, kKappaLo), kKappaHi));
		const float* m = o + 5 * j + 2;
		nrm[j]        = sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
		const bool flat = !(nrm[j] > 1e-6f); // read as +z, no gradient
		mu[j][0]      = flat ? 0.0f : m[0] / nrm[j];
		mu[j][1]      = flat ? 0.0f : m[1] / nrm[j];
		mu[j][2]      = flat ? 1.0f : m[2] / nrm[j];
		if (flat) nrm[j] = __int_as_float(0x7f800000);
		cs[j]         = mu[j][0] * d.x + mu[j][1] * d.y + mu[j][2] * d.z;
		const float lv = logf(kap[j]) - 1.8378770664093453f - log1pf(-expf(-2.0f * kap[j])) + kap[j] * (cs[j] - 1.0f);
		pv[j]         = pi[j] * expf(lv);
		q += pv[j];
	}
	const float qs = fmaxf(q, 1e-30f);
	loss           = -w * logf(qs);
	const float s  = -w * invN;
#pragma unroll
	for (int j = 0; j < kGuideLobes; ++j) {
		const float gamma = pv[j] / qs;
		g[5 * j]          = s * (gamma - pi[j]);
		const float e2    = expf(-2.0f * kap[j]);
		const float dl    = 1.0f / kap[j] - 2.0f * e2 / (1.0f - e2) + (cs[j] - 1.0f);
		g[5 * j + 1]      = live[j] ? s * gamma * dl * kap[j] : 0.0f;
		const float sg    = s * gamma * kap[j];
		const float gm[3] = { sg * d.x, sg * d.y, sg * d.z };
		const float proj  = gm[0] * mu[j][0] + gm[1] * mu[j][1] + gm[2] * mu[j][2];
#pragma unroll
		for (int a = 0; a < 3; ++a) g[5 * j + 2 + a] = (gm[a] - proj * mu[j][a]) / nrm[j];
	}
#pragma unroll
	for (int k = 5 * kGuideLobes; k < int(kOutW); ++k) g[k] = 0.0f;
}

__device__ __forceinline__ void initBarriers(uint32_t load, uint32_t mmaBar) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(load) : "memory");
	asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mmaBar) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void allocTmem(uint32_t slot, uint32_t cols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(cols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void freeTmem(uint32_t tmem, uint32_t cols) { asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory"); }
// the weight images by bulk copies of 4 KiB, all on one barrier
__device__ __forceinline__ void loadImages(uint32_t dst, const uint8_t* src, uint32_t bytes, uint32_t bar) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
	for (uint32_t o = 0; o < bytes; o += 4096u)
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst + o), "l"(src + o), "r"(4096u), "r"(bar) : "memory");
}

struct TrainArgs {
	const float* samples;
	uint32_t first, n;     // rows first .. first + n of the batch
	uint32_t total;        // samples held; row i reads sample (i * stride + offset) % total
	uint32_t stride, offset;
	const uint8_t* packed;
	const __half2* table;
	uint32_t tableLog2;
	Region region;
	float* wGrad;
	float* tGrad;
	float* loss;
	uint32_t* error;
};

__global__ void __launch_bounds__(128, 1) trainKernel(const __grid_constant__ TrainArgs A) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const uint32_t tid = threadIdx.x;
	uint8_t* X[4]      = { sm + kSX0, sm + kSX1, sm + kSX2, sm + kSX3 };
	uint8_t* DY        = sm + kSDY;
	uint8_t* DYT       = sm + kSDYT;
	uint8_t* XT        = sm + kSXT;
	uint64_t* bars     = reinterpret_cast<uint64_t*>(sm + kSBar);
	uint32_t* slot     = reinterpret_cast<uint32_t*>(sm + kSBar + 16);
	const uint32_t barLoad = sAddr(bars), barMma = sAddr(bars + 1);
	if (tid == 0) initBarriers(barLoad, barMma);
	if (tid < 32) allocTmem(sAddr(slot), 256);
	// the padded rows of the transposed gradient stay zero
	for (uint32_t i = tid; i < 32768u / 16u; i += 128u) reinterpret_cast<uint4*>(DYT)[i] = make_uint4(0, 0, 0, 0);
	stage();
	const uint32_t tmem = *slot;
	if (tid == 0) loadImages(sAddr(sm), A.packed, kPacked, barLoad);

	const uint32_t row = blockIdx.x * 128u + tid;
	const bool live    = row < A.n;
	float3 pos = make_float3(0, 0, 0), nrm = make_float3(0, 0, 0), dir = make_float3(0, 0, 1);
	float weight = 0.0f;
	float v[64];
	if (live) {
		const uint32_t s = uint32_t((uint64_t(A.first + row) * A.stride + A.offset) % A.total);
		const float* r   = A.samples + size_t(s) * kGuideSampleFloats;
		pos              = make_float3(r[0], r[1], r[2]);
		nrm              = make_float3(r[3], r[4], r[5]);
		dir              = make_float3(r[6], r[7], r[8]);
		weight           = r[9];
		encodeRow(A.table, A.tableLog2, A.region, pos, nrm, v);
	} else {
#pragma unroll
		for (int k = 0; k < int(kIn); ++k) v[k] = 0.0f;
	}
	storeRow<48>(X[0], tid, v, false);
	bool ok = waitBar(barLoad, 0);
	stage();
	uint32_t phase = 0;
	bool failed    = __syncthreads_or(!ok);
	// forward: layer l into TMEM columns 64 l
#pragma unroll
	for (int l = 0; l < 4; ++l) {
		if (failed) break;
		if (tid == 0) {
			mma(tmem + 64u * l, sAddr(X[l]), sAddr(sm + imgW(l)), nIn(l), nOut(l));
			commit(barMma);
		}
		ok = waitBar(barMma, phase);
		phase ^= 1u;
		if ((failed = __syncthreads_or(!ok))) break;
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		if (l < 3) {
			tload<64>(tmem, 64u * l, v);
			storeRow<64>(X[l + 1], tid, v, true);
			stage();
		}
	}
	float g[64];
	if (!failed) {
		tload<48>(tmem, 192u, v);
		float rowLoss = 0.0f;
		if (live) lossRow(v, dir, weight, 1.0f / float(A.n), g, rowLoss);
		else {
#pragma unroll
			for (int k = 0; k < 48; ++k) g[k] = 0.0f;
		}
		storeRow<48>(DY, tid, g, false);
		storeColumn<48>(DYT, tid, g);
		for (int o = 16; o > 0; o >>= 1) rowLoss += __shfl_xor_sync(0xFFFFFFFFu, rowLoss, o);
		if ((tid & 31u) == 0 && rowLoss != 0.0f) atomicAdd(A.loss, rowLoss / float(A.n));
		stage();
	}
	// backward: layer l's input gradient into columns 0.., its weight gradient into 64..
#pragma unroll
	for (int l = 3; l >= 0; --l) {
		if (failed) break;
		float xr[64];
		if (l == 0) readRow<48>(X[0], tid, xr);
		else readRow<64>(X[l], tid, xr);
		if (l == 0) storeColumn<48>(XT, tid, xr);
		else storeColumn<64>(XT, tid, xr);
		stage();
		if (tid == 0) {
			mma(tmem, sAddr(DY), sAddr(sm + imgWt(l)), nOut(l), nIn(l));
			mma(tmem + 64u, sAddr(DYT), sAddr(XT), 128u, nIn(l));
			commit(barMma);
		}
		ok = waitBar(barMma, phase);
		phase ^= 1u;
		if ((failed = __syncthreads_or(!ok))) break;
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		if (l == 0) tload<48>(tmem, 64u, v);
		else tload<64>(tmem, 64u, v);
		if (tid < nOut(l)) {
			float* dw = A.wGrad + wOff(l) + tid * nIn(l);
			for (uint32_t k = 0; k < nIn(l); ++k)
				if (v[k] != 0.0f) atomicAdd(dw + k, v[k]);
		}
		if (l == 0) tload<48>(tmem, 0u, v);
		else tload<64>(tmem, 0u, v);
		if (l > 0) {
#pragma unroll
			for (int k = 0; k < 64; ++k) g[k] = xr[k] > 0.0f ? v[k] : 0.0f;
			storeRow<64>(DY, tid, g, false);
			storeColumn<64>(DYT, tid, g);
		} else if (live) {
			float u[3];
			unitOf(A.region, pos, u);
			for (int lv = 0; lv < int(kLevels); ++lv) {
				uint32_t idx[8];
				float w[8];
				cornersAt(u, lv, A.tableLog2, idx, w);
				float* level = A.tGrad + (size_t(lv) << A.tableLog2) * 2u;
#pragma unroll
				for (int c = 0; c < 8; ++c) {
					atomicAdd(level + 2u * idx[c], w[c] * v[2 * lv]);
					atomicAdd(level + 2u * idx[c] + 1u, w[c] * v[2 * lv + 1]);
				}
			}
		}
		stage();
	}
	if (failed && tid == 0) atomicExch(A.error, 1u);
	__syncthreads();
	if (tid < 32) freeTmem(tmem, 256);
}

struct QueryArgs {
	const float* rows; // host-API rows: point, normal
	uint32_t n;
	GuideQueue queue;  // used where rows is null: the bounce's queue
	uint32_t capacity;
	const uint8_t* packed;
	const __half2* table;
	uint32_t tableLog2;
	Region region;
	float* lobes;
	uint32_t* error;
};

__global__ void __launch_bounds__(128) queryKernel(const __grid_constant__ QueryArgs A) {
	extern __shared__ __align__(1024) uint8_t sm[];
	const uint32_t tid = threadIdx.x;
	uint8_t* X0        = sm + kQX0;
	uint8_t* XA        = sm + kQXA;
	uint8_t* XB        = sm + kQXB;
	uint64_t* bars     = reinterpret_cast<uint64_t*>(sm + kQBar);
	uint32_t* slot     = reinterpret_cast<uint32_t*>(sm + kQBar + 16);
	const uint32_t barLoad = sAddr(bars), barMma = sAddr(bars + 1);
	const uint32_t n   = A.rows ? A.n : min(*A.queue.count, A.capacity);
	const uint32_t tiles = (n + 127u) / 128u;
	if (blockIdx.x >= tiles) return;
	if (tid == 0) initBarriers(barLoad, barMma);
	if (tid < 32) allocTmem(sAddr(slot), 128);
	stage();
	const uint32_t tmem = *slot;
	if (tid == 0) loadImages(sAddr(sm), A.packed, kForwardImages, barLoad);
	bool failed    = false;
	bool loaded    = false;
	uint32_t phase = 0;
	float v[64];
	for (uint32_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
		const uint32_t q = tile * 128u + tid;
		bool want        = q < n;
		float3 p = make_float3(0, 0, 0), nv = make_float3(0, 0, 0);
		if (want && A.rows) {
			const float* r = A.rows + size_t(q) * 6u;
			p              = make_float3(r[0], r[1], r[2]);
			nv             = make_float3(r[3], r[4], r[5]);
		} else if (want) {
			const kdn_hit& h = A.queue.hits[q];
			want             = h.kind != 0;
			if (want) {
				const Looks& L      = A.queue.looks;
				const uint32_t mat  = h.leaf < L.leafCount ? L.leafMaterial[h.leaf] : 0u;
				want                = guidable(L.materials[mat < A.queue.materialCount ? mat : 0u].kind);
				p                   = make_float3(h.point[0], h.point[1], h.point[2]);
				nv                  = make_float3(h.normal[0], h.normal[1], h.normal[2]);
				const kdn_ray& ray  = A.queue.rays[q];
				if (nv.x * ray.direction[0] + nv.y * ray.direction[1] + nv.z * ray.direction[2] >= 0.0f) nv = make_float3(-nv.x, -nv.y, -nv.z);
			}
		}
		if (want) encodeRow(A.table, A.tableLog2, A.region, p, nv, v);
		else {
#pragma unroll
			for (int k = 0; k < int(kIn); ++k) v[k] = 0.0f;
		}
		storeRow<48>(X0, tid, v, false);
		if (!loaded) {
			loaded = true;
			failed = __syncthreads_or(!waitBar(barLoad, 0));
		}
		stage();
		uint8_t* in[4]  = { X0, XA, XB, XA };
		uint8_t* out[3] = { XA, XB, XA };
#pragma unroll
		for (int l = 0; l < 4; ++l) {
			if (failed) break;
			if (tid == 0) {
				mma(tmem + 64u * (l & 1), sAddr(in[l]), sAddr(sm + imgW(l)), nIn(l), nOut(l));
				commit(barMma);
			}
			const bool ok = waitBar(barMma, phase);
			phase ^= 1u;
			if ((failed = __syncthreads_or(!ok))) break;
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			if (l < 3) {
				tload<64>(tmem, 64u * (l & 1), v);
				storeRow<64>(out[l], tid, v, true);
			} else {
				tload<48>(tmem, 64u, v);
			}
			stage();
		}
		if (!failed && want) {
			float L[kGuideLobeFloats];
			lobesOf(v, L);
			float* o = A.lobes + size_t(q) * kGuideLobeFloats;
#pragma unroll
			for (int k = 0; k < kGuideLobeFloats; ++k) o[k] = L[k];
		}
	}
	if (failed && tid == 0) atomicExch(A.error, 1u);
	__syncthreads();
	if (tid < 32) freeTmem(tmem, 128);
}

__global__ void adamKernel(float* p, float* g, float* m, float* v, size_t n, float lr, float c1, float c2, __half* half) {
	for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
		const float gi = g[i];
		g[i]           = 0.0f;
		const float mi = 0.9f * m[i] + 0.1f * gi;
		const float vi = 0.99f * v[i] + 0.01f * gi * gi;
		m[i]           = mi;
		v[i]           = vi;
		const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
		p[i]           = pi;
		if (half) half[i] = __float2half_rn(pi);
	}
}

__global__ void halfKernel(const float* p, __half* h, size_t n) {
	for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) h[i] = __float2half_rn(p[i]);
}

// the FP32 master weights into BF16 operand images (each matrix and its transpose)
__global__ void packKernel(const float* w, uint8_t* packed) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= kWeights) return;
	const int l        = i < 3072u ? 0 : i < 7168u ? 1 : i < 11264u ? 2 : 3;
	const uint32_t e   = i - wOff(l);
	const uint32_t r   = e / nIn(l), k = e % nIn(l);
	const __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
	*reinterpret_cast<__nv_bfloat16*>(packed + imgW(l) + imgAt(r, k, nIn(l)))   = b;
	*reinterpret_cast<__nv_bfloat16*>(packed + imgWt(l) + imgAt(k, r, nOut(l))) = b;
}

// a chunk's records into samples; the warp's finds compacted by ballot and prefix
// A record is kept where a hash of its path and vertex falls under keep (of
// 2^24): a frame with more records than the samples hold keeps an even share
// of every part of the frame, not its first pixels.
__global__ void gatherKernel(const GuideRecord* rec, const float4* radiance, uint32_t paths, float* samples, uint32_t* count, uint32_t capacity, uint32_t keepShare, uint32_t salt) {
	const uint32_t lane = threadIdx.x & 31u;
	for (uint32_t base = blockIdx.x * blockDim.x; base < paths; base += gridDim.x * blockDim.x) {
		const uint32_t p = base + threadIdx.x;
		const bool live  = p < paths;
		float total      = 0.0f;
		if (live) {
			const float4 R = radiance[p];
			total          = R.x + R.y + R.z + R.w;
		}
		for (int v = 0; v < kGuideDepth; ++v) {
			GuideRecord r {};
			float w   = 0.0f;
			bool keep = false;
			if (live) {
				r    = rec[size_t(p) * kGuideDepth + v];
				w    = (total - r.before) / r.reached;
				keep = isfinite(r.direction[0]) && isfinite(r.before) && r.reached > 0.0f && w > 0.0f && isfinite(w);
				uint32_t h = ((p * uint32_t(kGuideDepth) + uint32_t(v)) ^ salt) * 0x9E3779B1u;
				h ^= h >> 15;
				h *= 0x2C1B3C6Du;
				h ^= h >> 12;
				keep = keep && (h & 0xFFFFFFu) < keepShare;
			}
			const uint32_t mask = __ballot_sync(0xFFFFFFFFu, keep);
			if (mask == 0) continue;
			uint32_t first = 0;
			if (lane == 0) first = atomicAdd(count, uint32_t(__popc(mask)));
			first            = __shfl_sync(0xFFFFFFFFu, first, 0);
			const uint32_t s = first + uint32_t(__popc(mask & ((1u << lane) - 1u)));
			if (keep && s < capacity) {
				float* o = samples + size_t(s) * kGuideSampleFloats;
				o[0] = r.point[0], o[1] = r.point[1], o[2] = r.point[2];
				o[3] = r.normal[0], o[4] = r.normal[1], o[5] = r.normal[2];
				o[6] = r.direction[0], o[7] = r.direction[1], o[8] = r.direction[2];
				o[9] = w;
			}
		}
	}
}

// ---- host side ----

thread_local std::string tError;

kdn_status fail(const char* what, cudaError_t e) {
	tError = std::string(what) + ": " + cudaGetErrorString(e);
	return KDN_CUDA_ERROR;
}
#define GCHECK(call, what)                                   \
	do {                                                     \
		cudaError_t e_ = (call);                             \
		if (e_ != cudaSuccess) return fail((what), e_);      \
	} while (0)

size_t tableFloats(const kdn_guide* g) { return (size_t(kLevels) << g->tableLog2) * 2u; }

uint64_t splitmix(uint64_t& s) {
	uint64_t z = (s += 0x9E3779B97F4A7C15ull);
	z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
float uniform(uint64_t& s) { return float(double(splitmix(s) >> 11) * (1.0 / 9007199254740992.0)); }

TrainArgs trainArgs(kdn_guide* g) {
	TrainArgs a {};
	a.samples   = g->samples;
	a.packed    = g->packed;
	a.table     = reinterpret_cast<const __half2*>(g->tHalf);
	a.tableLog2 = g->tableLog2;
	for (int k = 0; k < 3; ++k) a.region.lo[k] = g->lo[k], a.region.hi[k] = g->hi[k];
	a.wGrad  = g->wGrad;
	a.tGrad  = g->tGrad;
	a.loss   = g->loss;
	a.error  = g->error;
	a.stride = 1;
	a.offset = 0;
	return a;
}

cudaError_t launchTrain(const TrainArgs& a, cudaStream_t s) {
	static std::once_flag once;
	static cudaError_t setup = cudaSuccess;
	std::call_once(once, [] { setup = cudaFuncSetAttribute(trainKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmem)); });
	if (setup != cudaSuccess) return setup;
	trainKernel<<<(a.n + 127u) / 128u, 128, kTrainSmem, s>>>(a);
	return cudaGetLastError();
}

cudaError_t launchQuery(const QueryArgs& a, uint32_t rowsMax, cudaStream_t s, int smCount) {
	static std::once_flag once;
	static cudaError_t setup = cudaSuccess;
	std::call_once(once, [] { setup = cudaFuncSetAttribute(queryKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kQuerySmem)); });
	if (setup != cudaSuccess) return setup;
	const uint32_t tiles = std::max(1u, (rowsMax + 127u) / 128u);
	const uint32_t grid  = std::min(tiles, uint32_t(std::max(1, smCount)) * 2u);
	queryKernel<<<grid, 128, kQuerySmem, s>>>(a);
	return cudaGetLastError();
}

// Adam over the weights and the table, then the BF16 images and the FP16 table
cudaError_t adamStep(kdn_guide* g, cudaStream_t s) {
	g->step += 1;
	const float c1 = float(1.0 - std::pow(0.9, double(g->step)));
	const float c2 = float(1.0 - std::pow(0.99, double(g->step)));
	adamKernel<<<(kWeights + 255) / 256, 256, 0, s>>>(g->weights, g->wGrad, g->wM, g->wV, kWeights, g->lr, c1, c2, nullptr);
	const size_t tf = tableFloats(g);
	adamKernel<<<std::max(1, g->smCount) * 8, 256, 0, s>>>(g->table, g->tGrad, g->tM, g->tV, tf, g->lr, c1, c2, g->tHalf);
	packKernel<<<(kWeights + 255) / 256, 256, 0, s>>>(g->weights, g->packed);
	return cudaGetLastError();
}

// steps of batch rows over the samples held, row i reading sample (i * stride + offset) % total
kdn_status trainOver(kdn_guide* g, uint32_t total, uint32_t batch, uint32_t steps, uint32_t stride, cudaStream_t s) {
	TrainArgs a = trainArgs(g);
	a.total     = total;
	a.stride    = stride;
	for (uint32_t k = 0; k < steps; ++k) {
		a.first  = uint32_t((uint64_t(k) * batch) % total);
		a.n      = std::min(batch, total);
		a.offset = 0;
		GCHECK(launchTrain(a, s), "guide train kernel");
		GCHECK(adamStep(g, s), "guide adam");
	}
	return KDN_OK;
}

uint32_t strideFor(uint32_t total) {
	// a stride prime to the count visits every sample once a pass, spread
	const uint32_t primes[] = { 1000003u, 999983u, 1048573u, 2147483647u };
	for (uint32_t p : primes)
		if (total % p != 0) return p % total == 0 ? 1u : p;
	return 1u;
}

kdn_status ensureSamples(kdn_guide* g, uint32_t n) {
	if (n <= g->capacity) return KDN_OK;
	if (g->samples) cudaFree(g->samples);
	g->samples  = nullptr;
	g->capacity = 0;
	GCHECK(cudaMalloc(&g->samples, size_t(n) * kGuideSampleFloats * sizeof(float)), "cudaMalloc guide samples");
	g->capacity = n;
	return KDN_OK;
}

kdn_status checkError(kdn_guide* g) {
	uint32_t e = 0;
	GCHECK(cudaMemcpy(&e, g->error, 4, cudaMemcpyDeviceToHost), "guide error flag");
	if (e != 0) {
		tError = "guide kernel reached its wait limit";
		cudaMemset(g->error, 0, 4);
		return KDN_TIMEOUT;
	}
	return KDN_OK;
}

} // namespace

int guideDevice(const kdn_guide* g) { return g->device; }

cudaError_t guideQueryQueue(kdn_guide* g, const GuideQueue& queue, uint32_t capacity, cudaStream_t stream, int smCount) {
	QueryArgs a {};
	a.rows      = nullptr;
	a.queue     = queue;
	a.capacity  = capacity;
	a.packed    = g->packed;
	a.table     = reinterpret_cast<const __half2*>(g->tHalf);
	a.tableLog2 = g->tableLog2;
	for (int k = 0; k < 3; ++k) a.region.lo[k] = g->lo[k], a.region.hi[k] = g->hi[k];
	a.lobes = queue.lobes;
	a.error = g->error;
	return launchQuery(a, capacity, stream, smCount);
}

cudaError_t guideGather(kdn_guide* g, const GuideRecord* records, const float4* radiance, uint32_t paths, uint64_t framePaths, uint32_t salt, cudaStream_t stream, int smCount) {
	const uint32_t blocks = std::min((paths + 255u) / 256u, uint32_t(std::max(1, smCount)) * 8u);
	// about half the vertices leave a record: keep an even share that fills the samples
	const double share    = std::min(1.0, double(g->capacity) / (0.5 * double(framePaths) * kGuideDepth));
	const uint32_t keep   = share >= 1.0 ? (1u << 24) : uint32_t(share * double(1u << 24));
	gatherKernel<<<std::max(1u, blocks), 256, 0, stream>>>(records, radiance, paths, g->samples, g->count, g->capacity, keep, salt);
	return cudaGetLastError();
}

kdn_status guideTrainGathered(kdn_guide* g, cudaStream_t stream) {
	uint32_t n = 0;
	GCHECK(cudaMemcpyAsync(&n, g->count, 4, cudaMemcpyDeviceToHost, stream), "guide sample count");
	GCHECK(cudaStreamSynchronize(stream), "guide sample count");
	n = std::min(n, g->capacity);
	GCHECK(cudaMemsetAsync(g->count, 0, 4, stream), "guide sample count");
	if (n == 0) return KDN_OK;
	const uint32_t steps = std::min(g->maxSteps, std::max(1u, (n + g->batch - 1u) / g->batch));
	kdn_status s         = trainOver(g, n, g->batch, steps, strideFor(n), stream);
	if (s != KDN_OK) return s;
	g->ready = true;
	return KDN_OK;
}

} // namespace kdn

using namespace kdn;

extern "C" {

const char* kdn_guide_last_error(void) { return tError.c_str(); }

kdn_status kdn_guide_open(int device, const kdn_guide_options* o, kdn_guide** out) {
	if (out == nullptr || o == nullptr) return KDN_BAD_ARG;
	*out = nullptr;
	if (o->table_log2 < 8 || o->table_log2 > 22 || !(o->learning_rate > 0.0f)) return KDN_BAD_ARG;
	for (int k = 0; k < 3; ++k)
		if (!(o->region_hi[k] > o->region_lo[k])) return KDN_BAD_ARG;
	GCHECK(cudaSetDevice(device), "cudaSetDevice");
	kdn_guide* g = new (std::nothrow) kdn_guide();
	if (g == nullptr) return KDN_OOM;
	g->device    = device;
	g->tableLog2 = o->table_log2;
	g->lr        = o->learning_rate;
	if (o->batch) g->batch = std::min<uint32_t>(std::max<uint32_t>(o->batch, 128u), 1u << 20);
	if (o->max_steps) g->maxSteps = o->max_steps;
	for (int k = 0; k < 3; ++k) g->lo[k] = o->region_lo[k], g->hi[k] = o->region_hi[k];
	cudaDeviceGetAttribute(&g->smCount, cudaDevAttrMultiProcessorCount, device);
	const size_t tf = tableFloats(g);
	auto grab       = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess && cudaMemset(*p, 0, bytes) == cudaSuccess; };
	bool ok = grab((void**)&g->weights, kWeights * 4) && grab((void**)&g->wGrad, kWeights * 4) && grab((void**)&g->wM, kWeights * 4) &&
	          grab((void**)&g->wV, kWeights * 4) && grab((void**)&g->table, tf * 4) && grab((void**)&g->tGrad, tf * 4) && grab((void**)&g->tM, tf * 4) &&
	          grab((void**)&g->tV, tf * 4) && grab((void**)&g->tHalf, tf * 2) && grab((void**)&g->packed, kPacked) && grab((void**)&g->loss, 4) &&
	          grab((void**)&g->error, 4) && grab((void**)&g->count, 4) && cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) == cudaSuccess;
	const uint32_t cap = o->sample_capacity ? o->sample_capacity : (1u << 24);
	if (ok) ok = ensureSamples(g, cap) == KDN_OK;
	if (!ok) {
		tError = "guide: device allocation failed";
		kdn_guide_close(g);
		return KDN_OOM;
	}
	// Xavier-uniform weights (the unused output rows zero), table in +-1e-4
	uint64_t seed = 0x5EEDull ^ (uint64_t(o->seed) << 17);
	std::vector<float> w(kWeights, 0.0f);
	for (int l = 0; l < 4; ++l) {
		const float a = std::sqrt(6.0f / float(nIn(l) + nOut(l)));
		for (uint32_t r = 0; r < nOut(l); ++r)
			for (uint32_t k = 0; k < nIn(l); ++k) w[wOff(l) + r * nIn(l) + k] = (l == 3 && r >= uint32_t(5 * kGuideLobes)) ? 0.0f : (2.0f * uniform(seed) - 1.0f) * a;
	}
	std::vector<float> t(tf);
	for (auto& x : t) x = (2.0f * uniform(seed) - 1.0f) * 1e-4f;
	kdn_status s = kdn_guide_set_params(g, w.data(), t.data());
	if (s != KDN_OK) {
		kdn_guide_close(g);
		return s;
	}
	*out = g;
	return KDN_OK;
}

kdn_status kdn_guide_close(kdn_guide* g) {
	if (g == nullptr) return KDN_BAD_ARG;
	cudaSetDevice(g->device);
	if (g->stream) cudaStreamSynchronize(g->stream);
	void* ptrs[] = { g->weights, g->wGrad, g->wM, g->wV, g->table, g->tGrad, g->tM, g->tV, g->tHalf, g->packed, g->loss, g->error, g->samples, g->count };
	for (void* p : ptrs)
		if (p) cudaFree(p);
	if (g->stream) cudaStreamDestroy(g->stream);
	delete g;
	return KDN_OK;
}

kdn_status kdn_guide_sizes(const kdn_guide* g, uint64_t* weights, uint64_t* table) {
	if (g == nullptr) return KDN_BAD_ARG;
	if (weights) *weights = kWeights;
	if (table) *table = tableFloats(g);
	return KDN_OK;
}

kdn_status kdn_guide_get_params(kdn_guide* g, float* weights, float* table) {
	if (g == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(g->lock);
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	GCHECK(cudaStreamSynchronize(g->stream), "guide stream");
	if (weights) GCHECK(cudaMemcpy(weights, g->weights, kWeights * 4, cudaMemcpyDeviceToHost), "guide weights");
	if (table) GCHECK(cudaMemcpy(table, g->table, tableFloats(g) * 4, cudaMemcpyDeviceToHost), "guide table");
	return KDN_OK;
}

kdn_status kdn_guide_set_params(kdn_guide* g, const float* weights, const float* table) {
	if (g == nullptr) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(g->lock);
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	const size_t tf = tableFloats(g);
	if (weights) GCHECK(cudaMemcpyAsync(g->weights, weights, kWeights * 4, cudaMemcpyHostToDevice, g->stream), "guide weights");
	if (table) GCHECK(cudaMemcpyAsync(g->table, table, tf * 4, cudaMemcpyHostToDevice, g->stream), "guide table");
	packKernel<<<(kWeights + 255) / 256, 256, 0, g->stream>>>(g->weights, g->packed);
	halfKernel<<<std::max(1, g->smCount) * 4, 256, 0, g->stream>>>(g->table, g->tHalf, tf);
	GCHECK(cudaGetLastError(), "guide pack");
	GCHECK(cudaStreamSynchronize(g->stream), "guide set params");
	return KDN_OK;
}

kdn_status kdn_guide_gradients(kdn_guide* g, const float* samples, uint32_t n, float* loss, float* dweights, float* dtable) {
	if (g == nullptr || samples == nullptr || n == 0 || n > (1u << 20)) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(g->lock);
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	kdn_status s = ensureSamples(g, n);
	if (s != KDN_OK) return s;
	const size_t tf = tableFloats(g);
	GCHECK(cudaMemcpyAsync(g->samples, samples, size_t(n) * kGuideSampleFloats * 4, cudaMemcpyHostToDevice, g->stream), "guide samples");
	GCHECK(cudaMemsetAsync(g->wGrad, 0, kWeights * 4, g->stream), "guide grads");
	GCHECK(cudaMemsetAsync(g->tGrad, 0, tf * 4, g->stream), "guide grads");
	GCHECK(cudaMemsetAsync(g->loss, 0, 4, g->stream), "guide loss");
	TrainArgs a = trainArgs(g);
	a.first     = 0;
	a.n         = n;
	a.total     = n;
	GCHECK(launchTrain(a, g->stream), "guide train kernel");
	GCHECK(cudaStreamSynchronize(g->stream), "guide train kernel");
	if ((s = checkError(g)) != KDN_OK) return s;
	if (loss) GCHECK(cudaMemcpy(loss, g->loss, 4, cudaMemcpyDeviceToHost), "guide loss");
	if (dweights) GCHECK(cudaMemcpy(dweights, g->wGrad, kWeights * 4, cudaMemcpyDeviceToHost), "guide grads");
	if (dtable) GCHECK(cudaMemcpy(dtable, g->tGrad, tf * 4, cudaMemcpyDeviceToHost), "guide grads");
	GCHECK(cudaMemset(g->wGrad, 0, kWeights * 4), "guide grads");
	GCHECK(cudaMemset(g->tGrad, 0, tf * 4), "guide grads");
	return KDN_OK;
}

kdn_status kdn_guide_train(kdn_guide* g, const float* samples, uint32_t n, uint32_t batch, uint32_t steps, float* last_loss) {
	if (g == nullptr || samples == nullptr || n == 0 || batch == 0 || batch > (1u << 20)) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(g->lock);
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	kdn_status s = ensureSamples(g, n);
	if (s != KDN_OK) return s;
	GCHECK(cudaMemcpyAsync(g->samples, samples, size_t(n) * kGuideSampleFloats * 4, cudaMemcpyHostToDevice, g->stream), "guide samples");
	if (steps == 0) steps = (n + batch - 1u) / batch;
	if (steps > 1) {
		if ((s = trainOver(g, n, batch, steps - 1, 1u, g->stream)) != KDN_OK) return s;
	}
	// the last step reports its loss
	GCHECK(cudaMemsetAsync(g->loss, 0, 4, g->stream), "guide loss");
	TrainArgs a = trainArgs(g);
	a.total     = n;
	a.first     = uint32_t((uint64_t(steps - 1) * batch) % n);
	a.n         = std::min(batch, n);
	GCHECK(launchTrain(a, g->stream), "guide train kernel");
	GCHECK(adamStep(g, g->stream), "guide adam");
	GCHECK(cudaStreamSynchronize(g->stream), "guide train");
	if ((s = checkError(g)) != KDN_OK) return s;
	if (last_loss) GCHECK(cudaMemcpy(last_loss, g->loss, 4, cudaMemcpyDeviceToHost), "guide loss");
	g->ready = true;
	return KDN_OK;
}

kdn_status kdn_guide_query(kdn_guide* g, const float* rows, uint32_t n, float* lobes) {
	if (g == nullptr || rows == nullptr || lobes == nullptr || n == 0 || n > (1u << 24)) return KDN_BAD_ARG;
	std::lock_guard<std::mutex> guard(g->lock);
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	float* dRows  = nullptr;
	float* dLobes = nullptr;
	GCHECK(cudaMallocAsync((void**)&dRows, size_t(n) * 6 * 4, g->stream), "guide query rows");
	GCHECK(cudaMallocAsync((void**)&dLobes, size_t(n) * kGuideLobeFloats * 4, g->stream), "guide query lobes");
	GCHECK(cudaMemcpyAsync(dRows, rows, size_t(n) * 6 * 4, cudaMemcpyHostToDevice, g->stream), "guide query rows");
	QueryArgs a {};
	a.rows      = dRows;
	a.n         = n;
	a.packed    = g->packed;
	a.table     = reinterpret_cast<const __half2*>(g->tHalf);
	a.tableLog2 = g->tableLog2;
	for (int k = 0; k < 3; ++k) a.region.lo[k] = g->lo[k], a.region.hi[k] = g->hi[k];
	a.lobes = dLobes;
	a.error = g->error;
	GCHECK(launchQuery(a, n, g->stream, g->smCount), "guide query kernel");
	GCHECK(cudaMemcpyAsync(lobes, dLobes, size_t(n) * kGuideLobeFloats * 4, cudaMemcpyDeviceToHost, g->stream), "guide query lobes");
	cudaFreeAsync(dRows, g->stream);
	cudaFreeAsync(dLobes, g->stream);
	GCHECK(cudaStreamSynchronize(g->stream), "guide query");
	return checkError(g);
}

kdn_status kdn_guide_clear_samples(kdn_guide* g) {
	if (g == nullptr) return KDN_BAD_ARG;
	GCHECK(cudaSetDevice(g->device), "cudaSetDevice");
	GCHECK(cudaMemset(g->count, 0, 4), "guide sample count");
	return KDN_OK;
}

int kdn_guide_ready(const kdn_guide* g) { return g != nullptr && g->ready ? 1 : 0; }

} // extern "C"
