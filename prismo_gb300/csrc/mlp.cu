// Surrogate network: an ensemble of small MLPs (in -> h -> h -> h -> out, SiLU)
// mapping coupler geometry to S-parameter spectra, trained on the device.
//
// Every matrix product of the forward pass, the backward pass and the weight
// gradient is one GEMM form, C[m][n] = sum_k A[m][k] B[n][k] with both operands
// bf16 and K-contiguous, accumulated in float32 on the tensor cores
// (mma.sync m16n8k16, bf16 x bf16 -> f32).  The layouts that make every product
// K-contiguous are kept by the epilogues, which write each activation and each
// back-propagated gradient twice (row-major and transposed):
//   forward   z_l = a_l W_l^T + b_l          A = a_l [B][K],   B = W_l  [N][K]
//   data grad g_{l-1} = (g_l W_l) * silu'(z) A = g_l [B][N],   B = W_l^T [K][N]
//   weight    dW_l = g_l^T a_l               A = g_l^T [N][B], B = a_l^T [K][B]
// Ensemble members run side by side on gridDim.z.  Parameters are float32
// masters updated by Adam; the bf16 copies W and W^T the GEMMs read are written
// by the same Adam kernel.
//
// Forward activations (and the network inputs) are kept as a pair of bf16 values
// a = a_hi + a_lo (a_lo = bf16(a - a_hi)), and each forward product is
// A_hi W + A_lo W: a single bf16 activation carries 8 significant bits, the pair
// about 16, so that inference is limited by the bf16 weights alone.  (At this
// model size the held-out surrogate error measured the same either way.)
// Weights stay bf16; the backward pass uses a_hi and bf16 gradients.
#include <cuda_bf16.h>

#include <vector>

#include "pc_internal.cuh"
#include "tcgen05.cuh"

namespace pc {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int GT = 64;   // CTA tile (M and N)
constexpr int GK = 32;   // K chunk
constexpr int GPAD = 8;  // smem row padding (bf16 elements)

enum { EP_HIDDEN = 0, EP_OUT = 1, EP_BWD = 2, EP_WGRAD = 3 };

struct GemmP {
    const bf16* A;
    const bf16* A2;  // low part of A (split forward products), same strides
    int64_t lda, sA;
    const bf16* B;
    int64_t ldb, sB;
    int M, N, K;
    const float* bias;
    int64_t sBias;
    float* outF;  // z (hidden), y (out), dW (wgrad)
    int64_t ldo, sO;
    const float* zprev;  // bwd: pre-activation of the layer below
    int64_t ldz, sZ;
    bf16* outB;  // activation / gradient, row-major
    bf16* outB2;  // low part of the activation (forward), same layout
    int64_t ldb2, sOB;
    bf16* outT;  // the same, transposed
    int64_t ldt, sOT;
};

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int MODE>
__device__ __forceinline__ void epilogue(const GemmP& p, int z, int m, int n, float acc) {
    if (m >= p.M || n >= p.N) return;
    if (MODE == EP_HIDDEN) {
        const float v = acc + p.bias[z * p.sBias + n];
        p.outF[z * p.sO + (int64_t)m * p.ldo + n] = v;
        const float av = v * sigm(v);
        const bf16 a = __float2bfloat16_rn(av);
        p.outB[z * p.sOB + (int64_t)m * p.ldb2 + n] = a;
        p.outB2[z * p.sOB + (int64_t)m * p.ldb2 + n] = __float2bfloat16_rn(av - __bfloat162float(a));
        p.outT[z * p.sOT + (int64_t)n * p.ldt + m] = a;
    } else if (MODE == EP_OUT) {
        p.outF[z * p.sO + (int64_t)m * p.ldo + n] = acc + p.bias[z * p.sBias + n];
    } else if (MODE == EP_BWD) {
        const float zz = p.zprev[z * p.sZ + (int64_t)m * p.ldz + n];
        const float s = sigm(zz);
        const bf16 g = __float2bfloat16_rn(acc * (s * (1.0f + zz * (1.0f - s))));
        p.outB[z * p.sOB + (int64_t)m * p.ldb2 + n] = g;
        p.outT[z * p.sOT + (int64_t)n * p.ldt + m] = g;
    } else {
        p.outF[z * p.sO + (int64_t)m * p.ldo + n] = acc;
    }
}

// 64x64 tile per CTA, 4 warps of 32x32; K in chunks of 32 staged in shared memory.
// SPLIT: A is the pair (A, A2) and the product is A B + A2 B.
template <int MODE, bool SPLIT>
__global__ void __launch_bounds__(128) mlp_gemm(GemmP p) {
    __shared__ __align__(16) bf16 As[GT][GK + GPAD];
    __shared__ __align__(16) bf16 As2[SPLIT ? GT : 1][GK + GPAD];
    __shared__ __align__(16) bf16 Bs[GT][GK + GPAD];
    const int z = blockIdx.z;
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    const bf16* A = p.A + z * p.sA;
    const bf16* A2 = SPLIT ? p.A2 + z * p.sA : nullptr;
    const bf16* B = p.B + z * p.sB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

    for (int k0 = 0; k0 < p.K; k0 += GK) {
        // 64 rows x 32 bf16 = 4 chunks of 16 bytes per row, per operand
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int c = tid + r * 128;
            const int row = c >> 2, col = (c & 3) * 8;
            uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0), va2 = make_uint4(0, 0, 0, 0);
            if (m0 + row < p.M) {
                va = *reinterpret_cast<const uint4*>(A + (int64_t)(m0 + row) * p.lda + k0 + col);
                if (SPLIT) va2 = *reinterpret_cast<const uint4*>(A2 + (int64_t)(m0 + row) * p.lda + k0 + col);
            }
            if (n0 + row < p.N) vb = *reinterpret_cast<const uint4*>(B + (int64_t)(n0 + row) * p.ldb + k0 + col);
            *reinterpret_cast<uint4*>(&As[row][col]) = va;
            if (SPLIT) *reinterpret_cast<uint4*>(&As2[row][col]) = va2;
            *reinterpret_cast<uint4*>(&Bs[row][col]) = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + g;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + j * 8 + g;
                bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * t]);
                bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
            if (SPLIT) {
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int r = wm + i * 16 + g;
                    af[i][0] = *reinterpret_cast<const uint32_t*>(&As2[r][kk + 2 * t]);
                    af[i][1] = *reinterpret_cast<const uint32_t*>(&As2[r + 8][kk + 2 * t]);
                    af[i][2] = *reinterpret_cast<const uint32_t*>(&As2[r][kk + 2 * t + 8]);
                    af[i][3] = *reinterpret_cast<const uint32_t*>(&As2[r + 8][kk + 2 * t + 8]);
                }
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + wm + i * 16 + g, n = n0 + wn + j * 8 + 2 * t;
            epilogue<MODE>(p, z, m, n, acc[i][j][0]);
            epilogue<MODE>(p, z, m, n + 1, acc[i][j][1]);
            epilogue<MODE>(p, z, m + 8, n, acc[i][j][2]);
            epilogue<MODE>(p, z, m + 8, n + 1, acc[i][j][3]);
        }
}

// The forward products on the 5th-generation tensor cores: a 128-row x 256-column
// output tile per CTA (8 warps), accumulated in tensor memory by tcgen05.mma
// (kind::f16: bf16 x bf16 -> f32, M 128, N 256, K 16 per instruction) issued by one
// thread.  K runs in chunks of 32 through a 3-stage ring: every thread copies its
// 16-byte pieces with cp.async into 8-row x 16-byte core matrices (no swizzle,
// K-major), and a stage is refilled once the tcgen05.commit of the MMAs that read
// it has arrived on its mbarrier.  SPLIT: the hi and lo activation tiles go through
// two MMAs into the same accumulator.  Epilogue: warps w and w + 4 share tensor-
// memory lanes 32(w%4)..+31 (one output row per thread) and split the columns;
// per 32-column slice, tcgen05.ld, bias (a lane shuffle) and SiLU once per
// element, the transposed bf16 copy written straight from that layout (each warp
// store covers 32 consecutive rows), the row-major outputs after a per-warp
// transpose through shared memory (row stride 36 floats: conflict-free 16-byte
// accesses) as 16-byte / 8-byte stores of 4 columns per lane.
constexpr int TC_M = 128, TC_N = 256, TC_K = 32, TC_NST = 3, TC_THREADS = 256;
constexpr uint32_t TC_LBO = 128;                // core matrices adjacent along K
constexpr uint32_t TC_SBO = (TC_K / 8) * 128;   // core matrices adjacent along M / N
constexpr int TC_A_BYTES = TC_M * TC_K * 2;     // 8 KB
constexpr int TC_B_BYTES = TC_N * TC_K * 2;     // 16 KB
constexpr int TC_SCR = 32 * 36;                 // floats of one transpose slice
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

template <bool SPLIT>
__host__ __device__ constexpr int tc_stage_bytes() {
    return (SPLIT ? 2 : 1) * TC_A_BYTES + TC_B_BYTES;
}
template <bool SPLIT>
__host__ __device__ constexpr int tc_smem_bytes() {
    return 1024 + TC_NST * tc_stage_bytes<SPLIT>();
}

// byte offset of element (row, k) of a K-major chunk in the core-matrix layout
__device__ __forceinline__ int cm_off(int row, int k) {
    return (row >> 3) * TC_SBO + (k >> 3) * TC_LBO + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const uint32_t a = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
    const uint32_t b = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
    return a | (b << 16);
}

template <int MODE, bool SPLIT>
__global__ void __launch_bounds__(TC_THREADS) mlp_gemm_tc(GemmP p, unsigned* status) {
    static_assert(!SPLIT || MODE == EP_HIDDEN || MODE == EP_OUT, "split operands in forward products only");
    constexpr int NSCR = MODE == EP_HIDDEN ? 2 : 1;  // pre-activation (+ activation) slices
    static_assert(TC_THREADS / 32 * NSCR * TC_SCR * 4 <= TC_NST * tc_stage_bytes<SPLIT>(),
                  "epilogue scratch fits the stages");
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* base = tsm + ((1024u - (smem_u32(tsm) & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base);            // [TC_NST]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + 64);     // allocated tensor-memory address
    unsigned char* stages = base + 1024;
    const int z = blockIdx.z;
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * TC_N;
    const bf16* A = p.A + z * p.sA;
    const bf16* A2 = SPLIT ? p.A2 + z * p.sA : nullptr;
    const bf16* B = p.B + z * p.sB;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nk = p.K / TC_K;

    if (warp == 0) tmem_alloc(tslot, TC_N);
    if (tid == 0) {
        for (int i = 0; i < TC_NST; ++i) mbar_init(&bars[i], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = idesc_bf16_f32(TC_M, TC_N);

    // chunk kc -> stage kc % TC_NST; kc >= nk commits an empty group
    auto load = [&](int kc) {
        if (kc < nk) {
            unsigned char* sA = stages + (kc % TC_NST) * tc_stage_bytes<SPLIT>();
            unsigned char* sB = sA + (SPLIT ? 2 : 1) * TC_A_BYTES;
            const int k0 = kc * TC_K;
            for (int q = tid; q < TC_M * 4; q += TC_THREADS) {
                const int row = q >> 2, kq = (q & 3) * 8;
                const bool valid = m0 + row < p.M;
                const int64_t src = (int64_t)(valid ? m0 + row : 0) * p.lda + k0 + kq;
                cp_async16(sA + cm_off(row, kq), A + src, valid);
                if (SPLIT) cp_async16(sA + TC_A_BYTES + cm_off(row, kq), A2 + src, valid);
            }
            for (int q = tid; q < TC_N * 4; q += TC_THREADS) {
                const int row = q >> 2, kq = (q & 3) * 8;
                cp_async16(sB + cm_off(row, kq), B + (int64_t)(n0 + row) * p.ldb + k0 + kq, true);
            }
        }
        cp_async_commit();
    };

    for (int kc = 0; kc < TC_NST - 1; ++kc) load(kc);
    bool ok = true;
    for (int kc = 0; kc < nk; ++kc) {
        cp_async_wait<TC_NST - 2>();  // this thread's pieces of chunk kc have landed
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            unsigned char* sA = stages + (kc % TC_NST) * tc_stage_bytes<SPLIT>();
            unsigned char* sB = sA + (SPLIT ? 2 : 1) * TC_A_BYTES;
#pragma unroll
            for (int kk = 0; kk < TC_K / 16; ++kk) {
                const uint64_t bd = smem_desc(sB + kk * 2 * TC_LBO, TC_LBO, TC_SBO);
                tc_mma_bf16(tmem, smem_desc(sA + kk * 2 * TC_LBO, TC_LBO, TC_SBO), bd, idesc, kc > 0 || kk > 0);
                if (SPLIT)
                    tc_mma_bf16(tmem, smem_desc(sA + TC_A_BYTES + kk * 2 * TC_LBO, TC_LBO, TC_SBO), bd, idesc, true);
            }
            tc_commit(&bars[kc % TC_NST]);
        }
        // refill the stage of chunk kc - 1 with chunk kc + TC_NST - 1 once its MMAs are done
        const int nx = kc + TC_NST - 1;
        if (nx < nk && kc >= 1 && ok)
            ok = mbar_wait_bounded(&bars[(kc - 1) % TC_NST], (uint32_t)(((kc - 1) / TC_NST) & 1), TC_WAIT_LIMIT);
        load(ok ? nx : nk);
    }
    // the last chunk's commit covers every MMA issued before it
    const int lb = (nk - 1) % TC_NST;
    const uint32_t lpar = (uint32_t)(((nk - 1) / TC_NST) & 1);
    if (ok) ok = mbar_wait_bounded(&bars[lb], lpar, TC_WAIT_LIMIT);
    ok = __syncthreads_and(ok);  // uniform: the epilogue's tcgen05.ld and __syncwarp need whole warps
    if (!ok) {
        if (tid == 0) atomicOr(status, PC_STATUS_TIMEOUT);
        // in-flight MMAs still read shared memory and write tensor memory: wait for them
        // once more (bounded) before tensor memory is released
        mbar_wait_bounded(&bars[lb], lpar, TC_WAIT_LIMIT);
    }
    cp_async_wait<0>();
    tc_fence_after();
    if (ok) {
        float* sx = reinterpret_cast<float*>(stages) + warp * NSCR * TC_SCR;  // this warp's slices
        float* sa = sx + TC_SCR;
        const int quarter = warp & 3, c0 = (warp >> 2) * (TC_N / 2);
        const int mw = m0 + quarter * 32;
        const bool rowv = mw + lane < p.M;
        const float* bias = p.bias + z * p.sBias;
        const int rr = lane >> 3, cq = (lane & 7) * 4;  // transposed phase: row in a group of 4, column quad
#pragma unroll 1
        for (int c = c0; c < c0 + TC_N / 2; c += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
            const int nb = n0 + c;
            if (MODE == EP_BWD || MODE == EP_WGRAD) {
                // lane = row: the accumulator slice to shared memory
#pragma unroll
                for (int j = 0; j < 32; j += 4)
                    *reinterpret_cast<float4*>(&sx[lane * 36 + j]) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                __syncwarp();
                // row-major: 8 lanes per row, 4 columns each (coalesced)
#pragma unroll
                for (int r0 = 0; r0 < 32; r0 += 4) {
                    const int r = r0 + rr;
                    const int64_t m = mw + r;
                    if (m >= p.M) continue;
                    float4 x = *reinterpret_cast<const float4*>(&sx[r * 36 + cq]);
                    if (MODE == EP_WGRAD) {
                        *reinterpret_cast<float4*>(&p.outF[z * p.sO + m * p.ldo + nb + cq]) = x;
                    } else {
                        // g = (g W) silu'(z): bf16 in both layouts, the same values as mma.sync's epilogue
                        const float4 zz = *reinterpret_cast<const float4*>(&p.zprev[z * p.sZ + m * p.ldz + nb + cq]);
                        float* xp = &x.x;
                        const float* zp = &zz.x;
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            const float sg = sigm(zp[t]);
                            xp[t] = __bfloat162float(__float2bfloat16_rn(xp[t] * (sg * (1.0f + zp[t] * (1.0f - sg)))));
                        }
                        *reinterpret_cast<uint2*>(&p.outB[z * p.sOB + m * p.ldb2 + nb + cq]) =
                            make_uint2(pack_bf16x2(x.x, x.y), pack_bf16x2(x.z, x.w));
                        *reinterpret_cast<float4*>(&sx[r * 36 + cq]) = x;
                    }
                }
                __syncwarp();
                if (MODE == EP_BWD && rowv) {  // lane = row again: the transposed copy
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        p.outT[z * p.sOT + (int64_t)(nb + j) * p.ldt + mw + lane] = __float2bfloat16_rn(sx[lane * 36 + j]);
                }
                __syncwarp();
                continue;
            }
            const float bn = bias[nb + lane];
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                float4 xv, av;
                float* xp = &xv.x;
                float* ap = &av.x;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float x = v[j + t] + __shfl_sync(0xffffffffu, bn, j + t);
                    xp[t] = x;
                    if (MODE == EP_HIDDEN) {
                        ap[t] = x * sigm(x);
                        if (rowv) p.outT[z * p.sOT + (int64_t)(nb + j + t) * p.ldt + mw + lane] =
                            __float2bfloat16_rn(ap[t]);
                    }
                }
                *reinterpret_cast<float4*>(&sx[lane * 36 + j]) = xv;
                if (MODE == EP_HIDDEN) *reinterpret_cast<float4*>(&sa[lane * 36 + j]) = av;
            }
            __syncwarp();
#pragma unroll
            for (int r0 = 0; r0 < 32; r0 += 4) {
                const int r = r0 + rr;
                const int64_t m = mw + r;
                if (m < p.M) {
                    const float4 x = *reinterpret_cast<const float4*>(&sx[r * 36 + cq]);
                    *reinterpret_cast<float4*>(&p.outF[z * p.sO + m * p.ldo + nb + cq]) = x;
                    if (MODE == EP_HIDDEN) {
                        const float4 a = *reinterpret_cast<const float4*>(&sa[r * 36 + cq]);
                        const uint2 hi = make_uint2(pack_bf16x2(a.x, a.y), pack_bf16x2(a.z, a.w));
                        const float l0 = a.x - __bfloat162float(__float2bfloat16_rn(a.x));
                        const float l1 = a.y - __bfloat162float(__float2bfloat16_rn(a.y));
                        const float l2 = a.z - __bfloat162float(__float2bfloat16_rn(a.z));
                        const float l3 = a.w - __bfloat162float(__float2bfloat16_rn(a.w));
                        const uint2 lo = make_uint2(pack_bf16x2(l0, l1), pack_bf16x2(l2, l3));
                        *reinterpret_cast<uint2*>(&p.outB[z * p.sOB + m * p.ldb2 + nb + cq]) = hi;
                        *reinterpret_cast<uint2*>(&p.outB2[z * p.sOB + m * p.ldb2 + nb + cq]) = lo;
                    }
                }
            }
            __syncwarp();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TC_N);
}

// x [z][B][din] float -> bf16 pair [z][B][kp] (hi, lo) and hi [z][kp][B] (member stride
// Bmax * kp), zero padded
__global__ void mlp_pack(const float* __restrict__ x, int din, int kp, int B, int Bmax, bf16* __restrict__ xb,
                         bf16* __restrict__ xb2, bf16* __restrict__ xt) {
    const int z = blockIdx.y;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B * kp; e += gridDim.x * blockDim.x) {
        const int b = e / kp, k = e - (e / kp) * kp;
        const float v = k < din ? x[((int64_t)z * B + b) * din + k] : 0.f;
        const bf16 h = __float2bfloat16_rn(v);
        xb[(int64_t)z * Bmax * kp + e] = h;
        xb2[(int64_t)z * Bmax * kp + e] = __float2bfloat16_rn(v - __bfloat162float(h));
        xt[(int64_t)z * Bmax * kp + (int64_t)k * B + b] = h;
    }
}

// mean-squared error over [B][N]; g = 2 (y - t) / (B N) as bf16 (both layouts).
// y, g, g^T have member stride Bmax * N; targets are dense [z][B][N].
__global__ void mlp_mse(const float* __restrict__ y, const float* __restrict__ tg, int B, int Bmax, int N,
                        bf16* __restrict__ g, bf16* __restrict__ gt, float* __restrict__ loss) {
    const int z = blockIdx.y;
    const int64_t off = (int64_t)z * Bmax * N;
    const float sc = 2.0f / ((float)B * (float)N);
    float acc = 0.f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < B * N; e += gridDim.x * blockDim.x) {
        const float d = y[off + e] - tg[(int64_t)z * B * N + e];
        acc += d * d;
        const int b = e / N, n = e - (e / N) * N;
        const bf16 h = __float2bfloat16_rn(sc * d);
        g[off + e] = h;
        gt[off + (int64_t)n * B + b] = h;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(&loss[z], acc / ((float)B * (float)N));
}

// bias gradient: db[n] = sum_b g^T[n][b], one warp per n (member stride Bmax * N)
__global__ void mlp_bias_grad(const bf16* __restrict__ gt, int N, int B, int Bmax, float* __restrict__ db,
                              int64_t sDb) {
    const int z = blockIdx.y;
    const int n = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (n >= N) return;
    const bf16* row = gt + (int64_t)z * Bmax * N + (int64_t)n * B;
    float s = 0.f;
    for (int b = threadIdx.x & 31; b < B; b += 32) s += __bfloat162float(row[b]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) db[z * sDb + n] = s;
}

struct LayerSeg {
    int64_t w_off, b_off;  // into the per-member parameter vector
    int n, k;              // weight [n][k] (k padded)
};

// Adam on the float32 masters; weight entries also refresh the bf16 W and W^T
struct AdamP {
    float* w;
    const float* g;
    float* m;
    float* v;
    int64_t P;
    float lr_t, b1, b2, eps;
    LayerSeg seg[4];
    bf16* wb[4];
    bf16* wt[4];
    int64_t swb[4];
};

__global__ void mlp_adam(AdamP a) {
    const int z = blockIdx.y;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.P; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = z * a.P + e;
        const float gr = a.g[o];
        const float m = a.b1 * a.m[o] + (1.f - a.b1) * gr;
        const float v = a.b2 * a.v[o] + (1.f - a.b2) * gr * gr;
        a.m[o] = m;
        a.v[o] = v;
        const float w = a.w[o] - a.lr_t * m / (sqrtf(v) + a.eps);
        a.w[o] = w;
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const LayerSeg& s = a.seg[l];
            const int64_t r = e - s.w_off;
            if (r >= 0 && r < (int64_t)s.n * s.k) {
                const int n = (int)(r / s.k), k = (int)(r - (r / s.k) * s.k);
                const bf16 h = __float2bfloat16_rn(w);
                a.wb[l][z * a.swb[l] + r] = h;
                a.wt[l][z * a.swb[l] + (int64_t)k * s.n + n] = h;
            }
        }
    }
}

// refresh the bf16 copies from the masters (after pc_mlp_set_params)
__global__ void mlp_sync_bf16(AdamP a) {
    const int z = blockIdx.y;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.P; e += (int64_t)gridDim.x * blockDim.x) {
        const float w = a.w[z * a.P + e];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const LayerSeg& s = a.seg[l];
            const int64_t r = e - s.w_off;
            if (r >= 0 && r < (int64_t)s.n * s.k) {
                const int n = (int)(r / s.k), k = (int)(r - (r / s.k) * s.k);
                const bf16 h = __float2bfloat16_rn(w);
                a.wb[l][z * a.swb[l] + r] = h;
                a.wt[l][z * a.swb[l] + (int64_t)k * s.n + n] = h;
            }
        }
    }
}

}  // namespace
}  // namespace pc

using namespace pc;

struct pc_mlp {
    int members = 0, max_batch = 0;
    int din = 0;
    int kp[4] = {}, nn[4] = {};  // per layer: padded input width, output width
    LayerSeg seg[4] = {};
    int64_t P = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    bf16* wb[4] = {};
    bf16* wt[4] = {};
    bf16 *xb = nullptr, *xb2 = nullptr, *xt = nullptr;
    float* z[3] = {};
    bf16* act[3] = {};   // inputs of layers 1..3 (high part)
    bf16* act2[3] = {};  // low part
    bf16* actT[3] = {};
    float* y = nullptr;
    bf16* gr[4] = {};    // gradients w.r.t. pre-activations of layers 0..3
    bf16* grT[4] = {};
    float* d_loss = nullptr;
    long long t = 0;     // Adam steps taken
    int tc = 2;          // products on tcgen05 (1), mma.sync (0), or by launch size (2)
    unsigned* d_status = nullptr;
    long long launches = 0;
    std::vector<void*> allocs;
};

namespace pc {
namespace {

template <typename T>
int mlp_alloc(pc_mlp* n, T** p, size_t count) {
    void* q = nullptr;
    PC_CUDA_CHECK(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    PC_CUDA_CHECK(cudaMemset(q, 0, std::max<size_t>(count, 1) * sizeof(T)));
    n->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return PC_OK;
}

AdamP adam_args(pc_mlp* n) {
    AdamP a{};
    a.w = n->w;
    a.g = n->g;
    a.m = n->m;
    a.v = n->v;
    a.P = n->P;
    for (int l = 0; l < 4; ++l) {
        a.seg[l] = n->seg[l];
        a.wb[l] = n->wb[l];
        a.wt[l] = n->wt[l];
        a.swb[l] = (int64_t)n->nn[l] * n->kp[l];
    }
    return a;
}

template <int MODE, bool SPLIT = false>
int gemm(pc_mlp* n, GemmP p, cudaStream_t s) {
    dim3 grd((p.N + GT - 1) / GT, (p.M + GT - 1) / GT, n->members);
    mlp_gemm<MODE, SPLIT><<<grd, 128, 0, s>>>(p);
    ++n->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

// tcgen05 takes a product on request (tc 1), or (tc 2) when its 128 x 256 tiles
// give the launch at least TC_MIN_CTAS CTAs: smaller products (a 256-row training
// batch gives 8) finish sooner as the 64 x 64 tiles of mma.sync.
constexpr int TC_MIN_CTAS = 64;
inline bool use_tc(const pc_mlp* n, const GemmP& p) {
    if (n->tc == 0) return false;
    if (n->tc == 1) return true;
    return (int64_t)(p.N / TC_N) * ((p.M + TC_M - 1) / TC_M) * n->members >= TC_MIN_CTAS;
}

// forward products (split activations): tcgen05 when the shape fits its tiles
template <int MODE>
int gemm_fwd(pc_mlp* n, GemmP p, cudaStream_t s) {
    // the epilogue stores 4 columns (16 bytes of float32) at a time: the output (a
    // caller's buffer for the last layer) and its strides must keep that aligned
    const bool aligned = ((uintptr_t)p.outF & 15) == 0 && p.ldo % 4 == 0 && p.sO % 4 == 0;
    if (!use_tc(n, p) || !aligned || p.N % TC_N != 0 || p.K % TC_K != 0) return gemm<MODE, true>(n, p, s);
    // at least 110 KB of shared memory: at most two CTAs per SM, so that their 2 x 256
    // tensor-memory columns fit the SM's 512 and no allocation ever waits
    constexpr int smem = tc_smem_bytes<true>() > 110 * 1024 ? tc_smem_bytes<true>() : 110 * 1024;
    static bool attr = false;
    if (!attr) {
        PC_CUDA_CHECK(cudaFuncSetAttribute(mlp_gemm_tc<MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    dim3 grd(p.N / TC_N, (p.M + TC_M - 1) / TC_M, n->members);
    mlp_gemm_tc<MODE, true><<<grd, TC_THREADS, smem, s>>>(p, n->d_status);
    ++n->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

// backward products (data gradient, weight gradient) on tcgen05 when the shape fits
template <int MODE>
int gemm_bwd(pc_mlp* n, GemmP p, cudaStream_t s) {
    const bool aligned = MODE == EP_WGRAD ? (((uintptr_t)p.outF & 15) == 0 && p.ldo % 4 == 0 && p.sO % 4 == 0)
                                          : (((uintptr_t)p.outB & 7) == 0 && p.ldb2 % 4 == 0 && p.sOB % 4 == 0 &&
                                             ((uintptr_t)p.zprev & 15) == 0 && p.ldz % 4 == 0 && p.sZ % 4 == 0);
    const bool operands = p.lda % 8 == 0 && p.ldb % 8 == 0 && p.sA % 8 == 0 && p.sB % 8 == 0;
    if (!use_tc(n, p) || !aligned || !operands || p.N % TC_N != 0 || p.K % TC_K != 0) return gemm<MODE>(n, p, s);
    constexpr int smem = tc_smem_bytes<false>() > 110 * 1024 ? tc_smem_bytes<false>() : 110 * 1024;
    static bool attr = false;
    if (!attr) {
        PC_CUDA_CHECK(cudaFuncSetAttribute(mlp_gemm_tc<MODE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    dim3 grd(p.N / TC_N, (p.M + TC_M - 1) / TC_M, n->members);
    mlp_gemm_tc<MODE, false><<<grd, TC_THREADS, smem, s>>>(p, n->d_status);
    ++n->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

// forward of every member on x [members][B][din]; leaves z, activations, y
int forward(pc_mlp* n, const float* x, int B, cudaStream_t s) {
    const int M = n->members;
    mlp_pack<<<dim3(std::min(1024, (B * n->kp[0] + 255) / 256), M), 256, 0, s>>>(x, n->din, n->kp[0], B, n->max_batch,
                                                                                 n->xb, n->xb2, n->xt);
    ++n->launches;
    for (int l = 0; l < 4; ++l) {
        GemmP p{};
        p.A = l == 0 ? n->xb : n->act[l - 1];
        p.A2 = l == 0 ? n->xb2 : n->act2[l - 1];
        p.lda = n->kp[l];
        p.sA = (int64_t)n->max_batch * n->kp[l];
        p.B = n->wb[l];
        p.ldb = n->kp[l];
        p.sB = (int64_t)n->nn[l] * n->kp[l];
        p.M = B;
        p.N = n->nn[l];
        p.K = n->kp[l];
        p.bias = n->w + n->seg[l].b_off;
        p.sBias = n->P;
        int rc;
        if (l < 3) {
            p.outF = n->z[l];
            p.ldo = n->nn[l];
            p.sO = (int64_t)n->max_batch * n->nn[l];
            p.outB = n->act[l];
            p.outB2 = n->act2[l];
            p.ldb2 = n->nn[l];
            p.sOB = (int64_t)n->max_batch * n->nn[l];
            p.outT = n->actT[l];
            p.ldt = B;
            p.sOT = (int64_t)n->max_batch * n->nn[l];
            rc = gemm_fwd<EP_HIDDEN>(n, p, s);
        } else {
            p.outF = n->y;
            p.ldo = n->nn[3];
            p.sO = (int64_t)n->max_batch * n->nn[3];
            rc = gemm_fwd<EP_OUT>(n, p, s);
        }
        if (rc) return rc;
    }
    return PC_OK;
}

// loss and gradients w.r.t. every parameter (into n->g)
int backward(pc_mlp* n, const float* tg, int B, float* loss, cudaStream_t s) {
    const int M = n->members;
    const int N3 = n->nn[3];
    mlp_mse<<<dim3(std::min(1024, (B * N3 + 255) / 256), M), 256, 0, s>>>(n->y, tg, B, n->max_batch, N3, n->gr[3],
                                                                          n->grT[3], loss);
    ++n->launches;
    for (int l = 3; l >= 0; --l) {
        // weight gradient: dW[n][k] = sum_b g^T[n][b] a^T[k][b]
        GemmP p{};
        p.A = n->grT[l];
        p.lda = B;
        p.sA = (int64_t)n->max_batch * n->nn[l];
        p.B = l == 0 ? n->xt : n->actT[l - 1];
        p.ldb = B;
        p.sB = (int64_t)n->max_batch * n->kp[l];
        p.M = n->nn[l];
        p.N = n->kp[l];
        p.K = B;
        p.outF = n->g + n->seg[l].w_off;
        p.ldo = n->kp[l];
        p.sO = n->P;
        int rc = gemm_bwd<EP_WGRAD>(n, p, s);
        if (rc) return rc;
        mlp_bias_grad<<<dim3((n->nn[l] + 7) / 8, M), 256, 0, s>>>(n->grT[l], n->nn[l], B, n->max_batch,
                                                                   n->g + n->seg[l].b_off, n->P);
        ++n->launches;
        if (l == 0) break;
        // data gradient into the layer below: g_{l-1} = (g_l W_l) * silu'(z_{l-1})
        GemmP q{};
        q.A = n->gr[l];
        q.lda = n->nn[l];
        q.sA = (int64_t)n->max_batch * n->nn[l];
        q.B = n->wt[l];
        q.ldb = n->nn[l];
        q.sB = (int64_t)n->nn[l] * n->kp[l];
        q.M = B;
        q.N = n->kp[l];
        q.K = n->nn[l];
        q.zprev = n->z[l - 1];
        q.ldz = n->nn[l - 1];
        q.sZ = (int64_t)n->max_batch * n->nn[l - 1];
        q.outB = n->gr[l - 1];
        q.ldb2 = n->nn[l - 1];
        q.sOB = (int64_t)n->max_batch * n->nn[l - 1];
        q.outT = n->grT[l - 1];
        q.ldt = B;
        q.sOT = (int64_t)n->max_batch * n->nn[l - 1];
        rc = gemm_bwd<EP_BWD>(n, q, s);
        if (rc) return rc;
    }
    return PC_OK;
}

}  // namespace
}  // namespace pc

extern "C" {

int pc_mlp_create(int32_t members, int32_t max_batch, const int32_t dims[5], pc_mlp** out) {
    if (!out || !dims || members <= 0 || members > 64 || max_batch <= 0 || max_batch % 32 != 0 ||
        max_batch > (1 << 20))
        return PC_ERR_INVALID;
    if (dims[0] <= 0 || dims[0] > 32) return PC_ERR_INVALID;
    for (int l = 1; l < 5; ++l)
        if (dims[l] <= 0 || dims[l] % 32 != 0 || dims[l] > 4096) return PC_ERR_INVALID;
    *out = nullptr;
    pc_mlp* n = new pc_mlp();
    n->members = members;
    n->max_batch = max_batch;
    n->din = dims[0];
    int64_t off = 0;
    for (int l = 0; l < 4; ++l) {
        n->kp[l] = l == 0 ? 32 : dims[l];
        n->nn[l] = dims[l + 1];
        n->seg[l].n = n->nn[l];
        n->seg[l].k = n->kp[l];
        n->seg[l].w_off = off;
        off += (int64_t)n->nn[l] * n->kp[l];
        n->seg[l].b_off = off;
        off += n->nn[l];
    }
    n->P = off;
    const size_t Mb = (size_t)members, B = (size_t)max_batch;
    int rc = mlp_alloc(n, &n->w, Mb * off) || mlp_alloc(n, &n->g, Mb * off) || mlp_alloc(n, &n->m, Mb * off) ||
             mlp_alloc(n, &n->v, Mb * off) || mlp_alloc(n, &n->xb, Mb * B * 32) || mlp_alloc(n, &n->xb2, Mb * B * 32) ||
             mlp_alloc(n, &n->xt, Mb * B * 32) ||
             mlp_alloc(n, &n->y, Mb * B * n->nn[3]) || mlp_alloc(n, &n->d_loss, Mb) ||
             mlp_alloc(n, &n->d_status, 1);
    for (int l = 0; l < 4 && !rc; ++l) {
        rc = mlp_alloc(n, &n->wb[l], Mb * n->nn[l] * n->kp[l]) || mlp_alloc(n, &n->wt[l], Mb * n->nn[l] * n->kp[l]) ||
             mlp_alloc(n, &n->gr[l], Mb * B * n->nn[l]) || mlp_alloc(n, &n->grT[l], Mb * B * n->nn[l]);
        if (!rc && l < 3)
            rc = mlp_alloc(n, &n->z[l], Mb * B * n->nn[l]) || mlp_alloc(n, &n->act[l], Mb * B * n->nn[l]) ||
                 mlp_alloc(n, &n->act2[l], Mb * B * n->nn[l]) || mlp_alloc(n, &n->actT[l], Mb * B * n->nn[l]);
    }
    if (rc) {
        pc_mlp_destroy(n);
        return PC_ERR_CUDA;
    }
    *out = n;
    return PC_OK;
}

int64_t pc_mlp_param_count(const pc_mlp* n) { return n ? n->P : PC_ERR_INVALID; }

int pc_mlp_param_layout(const pc_mlp* n, int32_t layer, int64_t out[4]) {
    if (!n || !out || layer < 0 || layer > 3) return PC_ERR_INVALID;
    out[0] = n->seg[layer].w_off;
    out[1] = n->seg[layer].b_off;
    out[2] = n->seg[layer].n;
    out[3] = n->seg[layer].k;
    return PC_OK;
}

int pc_mlp_set_params(pc_mlp* n, const float* host) {
    if (!n || !host) return PC_ERR_INVALID;
    const size_t bytes = (size_t)n->members * n->P * sizeof(float);
    PC_CUDA_CHECK(cudaMemcpy(n->w, host, bytes, cudaMemcpyHostToDevice));
    PC_CUDA_CHECK(cudaMemset(n->m, 0, bytes));
    PC_CUDA_CHECK(cudaMemset(n->v, 0, bytes));
    n->t = 0;
    AdamP a = adam_args(n);
    mlp_sync_bf16<<<dim3(std::min<int64_t>(1024, (n->P + 255) / 256), n->members), 256>>>(a);
    ++n->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    PC_CUDA_CHECK(cudaDeviceSynchronize());
    return PC_OK;
}

int pc_mlp_get_params(const pc_mlp* n, float* host) {
    if (!n || !host) return PC_ERR_INVALID;
    PC_CUDA_CHECK(cudaMemcpy(host, n->w, (size_t)n->members * n->P * sizeof(float), cudaMemcpyDeviceToHost));
    return PC_OK;
}

int pc_mlp_get_grads(const pc_mlp* n, float* host) {
    if (!n || !host) return PC_ERR_INVALID;
    PC_CUDA_CHECK(cudaMemcpy(host, n->g, (size_t)n->members * n->P * sizeof(float), cudaMemcpyDeviceToHost));
    return PC_OK;
}

int pc_mlp_forward(pc_mlp* n, const float* d_x, int32_t batch, float* d_y, void* stream) {
    if (!n || !d_x || !d_y || batch <= 0 || batch > n->max_batch) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = forward(n, d_x, batch, s);
    if (rc) return rc;
    const size_t row = (size_t)n->nn[3] * sizeof(float);
    PC_CUDA_CHECK(cudaMemcpy2DAsync(d_y, (size_t)batch * row, n->y, (size_t)n->max_batch * row, (size_t)batch * row,
                                    n->members, cudaMemcpyDeviceToDevice, s));
    return PC_OK;
}

int pc_mlp_gradients(pc_mlp* n, const float* d_x, const float* d_t, int32_t batch, float* d_loss, void* stream) {
    if (!n || !d_x || !d_t || batch <= 0 || batch > n->max_batch || batch % 32 != 0) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PC_CUDA_CHECK(cudaMemsetAsync(n->d_loss, 0, n->members * sizeof(float), s));
    int rc = forward(n, d_x, batch, s);
    if (rc) return rc;
    rc = backward(n, d_t, batch, n->d_loss, s);
    if (rc) return rc;
    if (d_loss)
        PC_CUDA_CHECK(
            cudaMemcpyAsync(d_loss, n->d_loss, n->members * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return PC_OK;
}

int pc_mlp_train_step(pc_mlp* n, const float* d_x, const float* d_t, int32_t batch, float lr, float beta1,
                      float beta2, float eps, float* d_loss, void* stream) {
    if (!n || !(lr > 0) || !(beta1 >= 0 && beta1 < 1) || !(beta2 >= 0 && beta2 < 1) || !(eps > 0))
        return PC_ERR_INVALID;
    int rc = pc_mlp_gradients(n, d_x, d_t, batch, d_loss, stream);
    if (rc) return rc;
    ++n->t;
    AdamP a = adam_args(n);
    a.b1 = beta1;
    a.b2 = beta2;
    a.eps = eps;
    a.lr_t = (float)(lr * sqrt(1.0 - pow((double)beta2, (double)n->t)) / (1.0 - pow((double)beta1, (double)n->t)));
    mlp_adam<<<dim3(std::min<int64_t>(1024, (n->P + 255) / 256), n->members), 256, 0, (cudaStream_t)stream>>>(a);
    ++n->launches;
    PC_CUDA_CHECK(cudaGetLastError());
    return PC_OK;
}

int64_t pc_mlp_launch_count(const pc_mlp* n) { return n ? n->launches : PC_ERR_INVALID; }

int pc_mlp_set_tensor_path(pc_mlp* n, int32_t tcgen05) {
    if (!n || tcgen05 < 0 || tcgen05 > 2) return PC_ERR_INVALID;
    n->tc = tcgen05;
    return PC_OK;
}

int pc_mlp_status(pc_mlp* n, uint32_t* flags, void* stream) {
    if (!n || !flags) return PC_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PC_CUDA_CHECK(cudaMemcpyAsync(flags, n->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    PC_CUDA_CHECK(cudaStreamSynchronize(s));
    return PC_OK;
}

void pc_mlp_destroy(pc_mlp* n) {
    if (!n) return;
    for (void* p : n->allocs) cudaFree(p);
    delete n;
}

}  // extern "C"
