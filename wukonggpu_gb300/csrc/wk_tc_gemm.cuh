// The estimator's GEMM on the 5th-generation tensor cores (sm_100 family):
// C[M x N] fp32 = A[M x K] . B[N x K]^T (+ bias[n]), A and B bf16 row-major
// (K contiguous), FP32 accumulation in tensor memory (TMEM).
//
// One CTA of 4 warps computes a 128 x BN tile (BN = 32, 64, 128 or 256: one
// MMA shape); the grid is M tiles x N / BN.  K is walked in slabs of 64 bf16 -- one
// 128-byte row of the 128 B swizzle -- through kStages shared-memory stages:
//   - thread 0 (the producer) loads each slab's A box (64 x 128) and B box
//     (64 x BN) with TMA (cp.async.bulk.tensor.2d, 128 B swizzle; rows past M
//     and columns past K read as zero), completing on the stage's "full"
//     mbarrier, once the stage's "empty" mbarrier says its last products ran;
//   - thread 32 (the MMA issuer) waits for "full", issues the slab's
//     tcgen05.mma (kind::f16, 128 x BN x 16 each) from shared-memory
//     descriptors and commits them to the stage's "empty" mbarrier;
//   - after the last commit, warp w reads TMEM lanes 32w..32w+31 (rows) in
//     32-column chunks with tcgen05.ld and runs the epilogue the template
//     names (EpiArgs):
//       kEpiStore:   C = acc (+ bias), staged in shared memory (the pipeline
//                    stages are free by then) and written as whole rows of
//                    float4, so a store instruction covers 4 rows x 128 B;
//       kEpiGeluFwd: the same C (the pre-activation Z), and H = GELU(Z) in
//                    bf16, row-major and transposed (zero for rows >= m_real);
//       kEpiGeluBwd: dZ = acc * GELU'(Z) in bf16, row-major and transposed
//                    (zero for rows >= m_real), and the column sums of the
//                    rounded dZ added into colsum[] -- C is not written.
// Every mbarrier wait is bounded.  A wait that runs out sets bit 2 of *err and
// stops the pipeline: the producer waits (bounded) for the copies it issued
// and the issuer for the last commit of the products it issued.  If those
// drain waits also run out, work may still be in flight, so the CTA sets bit
// 3 as well and exits without freeing its TMEM columns -- a unit still
// writing them must not find them given to another CTA.  The host then
// refuses every later call on the estimator (the TMEM and the device state
// are no longer trusted); nothing is reused.
#pragma once

#include <cstdint>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace wk {
namespace tc {

constexpr int kTM = 128;            // tile rows = MMA M
constexpr int kSlab = 64;           // K elements per stage (128 B rows)
constexpr int kStages = 4;
constexpr int kThreads = 128;
constexpr int kEpiPitch = 36;       // floats per staged output row: rows 16 B apart modulo 128 B
constexpr long kWaitIters = 1l << 22;

enum { kEpiStore = 0, kEpiGeluFwd = 1, kEpiGeluBwd = 2 };

// The epilogue's extra operands (unused by kEpiStore).  Rows below m_store get
// h / ht written (row-major with ld ldh, transposed with ld ldt); rows below
// m_real carry values, the rest zeros.
struct EpiArgs {
    int m_real = 0, m_store = 0;
    __nv_bfloat16 *h = nullptr;
    int ldh = 0;
    __nv_bfloat16 *ht = nullptr;
    int ldt = 0;
    const float *z = nullptr;   // kEpiGeluBwd: the layer's pre-activation (ld ldz)
    int ldz = 0;
    float *colsum = nullptr;    // kEpiGeluBwd: column sums of dZ are added here
};

// The estimator's activation, exact GELU: x Phi(x), and its derivative
// Phi(x) + x phi(x) (Phi, phi the standard normal CDF and density).
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128 B swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);   // start address / 16
    d |= (uint64_t)1 << 16;                   // leading byte offset (not used by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: the next group of 8 rows
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // 128 B swizzle
    return d;
}

// instruction descriptor of kind::f16: BF16 A and B, FP32 D, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    uint32_t done = 0;
    for (long it = 0; it < kWaitIters && !done; ++it)
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
    return done != 0;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(mbar) : "memory");
}

// 32 consecutive fp32 columns of the warp's 32 TMEM lanes: lane i gets row i
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// C must be 16 B aligned with ldc a multiple of 4, and bias (if any) 16 B
// aligned; h (and z) 16 B aligned with ldh (ldz) a multiple of 8 (4).
template <int BN, int EPI>
__global__ void __launch_bounds__(kThreads)
gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               float *__restrict__ C, int ldc, int M, int K, const float *__restrict__ bias, int *err,
               const EpiArgs ea) {
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "tile width: an MMA N and a TMEM allocation");
    constexpr uint32_t kABytes = kTM * 128, kBBytes = BN * 128, kStage = kABytes + kBBytes;
    static_assert(4 * 32 * kEpiPitch * 4 <= kStage, "the output staging fits in stage 0");
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) uint64_t s_full[kStages], s_empty[kStages];
    __shared__ volatile int s_fail;
    __shared__ volatile int s_inflight;   // a drain wait ran out: copies or products may be in flight
    // 128 B swizzle: stage bases 1024 B aligned
    unsigned char *sm = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * BN;
    const int nslab = (K + kSlab - 1) / kSlab;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&s_tmem)), "r"((uint32_t)BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (t == 0) {
        s_fail = 0;
        s_inflight = 0;
        for (int i = 0; i < kStages; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_empty[i])));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    // slab j lives in stage j % kStages as that stage's use u = j / kStages; each
    // barrier completes once per use, so the wait for use u is parity u % 2
    if (t == 0) {
        int issued = 0;
        for (int j = 0; j < nslab; ++j) {
            const int s = j % kStages, u = j / kStages;
            if (u > 0 && !mbar_wait(smem_u32(&s_empty[s]), (uint32_t)((u - 1) & 1))) {
                s_fail = 1;
                break;
            }
            const uint32_t a = smem_u32(sm + s * kStage), b = a + kABytes, fb = smem_u32(&s_full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kStage) : "memory");
            tma_load_2d(a, &tmA, j * kSlab, m0, fb);
            tma_load_2d(b, &tmB, j * kSlab, n0, fb);
            issued = j + 1;
        }
        // every copy in flight lands before the CTA can leave (immediate when all were consumed)
        for (int j = issued > kStages ? issued - kStages : 0; j < issued; ++j)
            if (!mbar_wait(smem_u32(&s_full[j % kStages]), (uint32_t)((j / kStages) & 1))) {
                s_fail = 1;
                s_inflight = 1;
                break;
            }
    } else if (t == 32) {
        int committed = 0;
        for (int sl = 0; sl < nslab; ++sl) {
            const int s = sl % kStages;
            if (!mbar_wait(smem_u32(&s_full[s]), (uint32_t)((sl / kStages) & 1))) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ad = smem_u32(sm + s * kStage), bd = ad + kABytes;
            const int ksteps = (K - sl * kSlab) >= kSlab ? kSlab / 16 : (K - sl * kSlab + 15) / 16;
            for (int kk = 0; kk < ksteps; ++kk) {
                const uint32_t acc = (sl > 0 || kk > 0) ? 1u : 0u;
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                             ::"r"(tmem), "l"(sw128_desc(ad + kk * 32)), "l"(sw128_desc(bd + kk * 32)),
                               "r"(idesc_bf16(kTM, BN)), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&s_empty[s])) : "memory");
            committed = sl + 1;
        }
        // the last commit covers every product issued: they complete before TMEM is read or freed
        if (committed > 0) {
            const int c = committed - 1;
            if (!mbar_wait(smem_u32(&s_empty[c % kStages]), (uint32_t)((c / kStages) & 1))) {
                s_fail = 1;
                s_inflight = 1;
            }
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail && nslab > 0) {
        // every copy landed and every product ran: stage 0 is free for the output rows
        float *stg = reinterpret_cast<float *>(sm) + warp * 32 * kEpiPitch;
        const int q = lane & 7;
        const int myrow = m0 + warp * 32 + lane;   // the row of this lane's TMEM lane
        for (int c0 = 0; c0 < BN; c0 += 32) {
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
            const int cb = n0 + c0;   // the chunk's first column
            float4 *mine = reinterpret_cast<float4 *>(stg + lane * kEpiPitch);
            if constexpr (EPI != kEpiGeluBwd) {
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    mine[i] = make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]),
                                          __uint_as_float(r[4 * i + 2]), __uint_as_float(r[4 * i + 3]));
                __syncwarp();
                const int col = cb + q * 4;
                const float4 bv = bias ? *reinterpret_cast<const float4 *>(bias + col) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int rr = i * 4 + (lane >> 3);
                    const int row = m0 + warp * 32 + rr;
                    float4 v = *reinterpret_cast<const float4 *>(stg + rr * kEpiPitch + q * 4);
                    v.x += bv.x; v.y += bv.y; v.z += bv.z; v.w += bv.w;
                    if (row < M) *reinterpret_cast<float4 *>(C + (size_t)row * ldc + col) = v;
                }
                __syncwarp();
            }
            if constexpr (EPI == kEpiGeluFwd || EPI == kEpiGeluBwd) {
                // this lane's row of the chunk: 32 values in bf16
                __nv_bfloat16 hv[32];
                if constexpr (EPI == kEpiGeluFwd) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const float zv = __uint_as_float(r[i]) + (bias ? bias[cb + i] : 0.f);
                        hv[i] = __float2bfloat16(myrow < ea.m_real ? gelu(zv) : 0.f);
                    }
                } else {
                    float zr[32] = {};
                    if (myrow < ea.m_real) {
                        const float4 *zp = reinterpret_cast<const float4 *>(ea.z + (size_t)myrow * ea.ldz + cb);
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float4 z4 = zp[i];
                            zr[4 * i] = z4.x; zr[4 * i + 1] = z4.y; zr[4 * i + 2] = z4.z; zr[4 * i + 3] = z4.w;
                        }
                    }
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        hv[i] = __float2bfloat16(myrow < ea.m_real ? __uint_as_float(r[i]) * gelu_grad(zr[i]) : 0.f);
                    // column sums of the rounded values: rows staged in shared memory, lane i sums column i
                    float *mrow = stg + lane * kEpiPitch;
#pragma unroll
                    for (int i = 0; i < 32; ++i) mrow[i] = __bfloat162float(hv[i]);
                    __syncwarp();
                    float cs = 0.f;
#pragma unroll 8
                    for (int rr = 0; rr < 32; ++rr) cs += stg[rr * kEpiPitch + lane];
                    if (cs != 0.f) atomicAdd(ea.colsum + cb + lane, cs);
                    __syncwarp();
                }
                if (myrow < ea.m_store) {
                    // element 2k at the lower address: the low half of word k
                    uint32_t w[16];
#pragma unroll
                    for (int k = 0; k < 16; ++k)
                        w[k] = (uint32_t)__bfloat16_as_ushort(hv[2 * k]) |
                               ((uint32_t)__bfloat16_as_ushort(hv[2 * k + 1]) << 16);
                    uint4 *hp = reinterpret_cast<uint4 *>(ea.h + (size_t)myrow * ea.ldh + cb);
#pragma unroll
                    for (int i = 0; i < 4; ++i) hp[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
#pragma unroll
                    for (int i = 0; i < 32; ++i) ea.ht[(size_t)(cb + i) * ea.ldt + myrow] = hv[i];
                }
            }
        }
    } else if (s_fail && t == 0) {
        atomicOr(err, s_inflight ? (4 | 8) : 4);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // products still in flight may write these columns: they stay allocated
    if (warp == 0 && !s_inflight) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN));
    }
}

inline size_t smem_bytes(int BN) { return kStages * ((size_t)kTM * 128 + (size_t)BN * 128) + 1024; }

// 2-D tensor map of a row-major bf16 matrix (rows x cols, row pitch ld elements,
// 16 B aligned): boxes of 64 columns x box_rows rows, 128 B swizzle, zero outside.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        // the entry point as CUDA 12.0 introduced it (its signature has not changed since)
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

inline bool make_map(CUtensorMap *map, const void *base, uint64_t rows, uint64_t cols, uint64_t ld,
                     uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || ((uintptr_t)base & 15u) || ((ld * 2) & 15u)) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kSlab, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc
}  // namespace wk
