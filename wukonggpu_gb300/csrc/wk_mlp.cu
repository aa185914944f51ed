// The learned cardinality estimator: an MLP trained and evaluated by
// hand-written BF16 tensor-core kernels.
//
// Model: x = [48 pattern features | 32-d embedding of the predicate] (80)
//        -> 256 -> 256 -> 256 (GELU after each) -> 1
// It predicts log(1 + rows) of the table after a pattern is applied.  Weights
// and activations are BF16, every product accumulates in FP32 in tensor
// memory on the 5th-generation tensor cores (tcgen05.mma with TMA-staged
// operands, wk_tc_gemm.cuh), and the optimiser is FP32 Adam over FP32 master
// weights whose BF16 copies are refreshed after each step.
//
// One GEMM kernel does all products: C[M x N] = A[M x K] . B[N x K]^T with A
// and B row-major (K contiguous), which is the natural form for the forward
// product (X . W^T), for the input gradient (dZ . W, with W^T kept as a BF16
// copy) and for the weight gradient (dZ^T . X, with the transposed
// activations written by the forward pass).  Dimensions are padded: M and N
// to multiples of 64, K to multiples of 16; padding is zero.  The hidden
// layers' activation runs in the GEMM's epilogue: the forward product writes
// GELU(Z) in bf16 (row-major and transposed) beside Z, and the input-gradient
// product of the layer above writes dZ = dH * GELU'(Z) with the bias
// gradient (its column sums), so dH itself is never stored.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "wk_runtime.h"
#include "wk_tc_gemm.cuh"

namespace wk {
namespace mlp {

constexpr int kIn = 48;       // pattern features
constexpr int kEmb = 32;      // predicate embedding
constexpr int kX = kIn + kEmb;   // 80
constexpr int kH = 256;
constexpr int kOutPad = 64;   // output layer padded to one GEMM tile
constexpr int kXPadN = 128;   // W1^T rows padded (dX GEMM has N = 80 -> 128)
constexpr float kB1 = 0.9f, kB2 = 0.999f;   // Adam moment decay rates

// ------------------------------------------------------------ elementwise
// X0 [Mp x 80] bf16 = [feats | emb[pid]] for real rows, 0 for padding
__global__ void build_input_kernel(const float *__restrict__ feats, const int32_t *__restrict__ pids, int M, int Mp,
                                   const float *__restrict__ emb, int n_ids, __nv_bfloat16 *__restrict__ X0,
                                   __nv_bfloat16 *__restrict__ X0t) {
    const int64_t n = (int64_t)Mp * kX;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / kX), c = (int)(i % kX);
        float v = 0.f;
        if (r < M) {
            if (c < kIn) v = feats[(size_t)r * kIn + c];
            else {
                int p = pids[r];
                p = p < 0 ? 0 : (p > n_ids ? n_ids : p);
                v = emb[(size_t)p * kEmb + (c - kIn)];
            }
        }
        const __nv_bfloat16 bv = __float2bfloat16(v);
        X0[i] = bv;
        X0t[(size_t)c * Mp + r] = bv;
    }
}

// column sums of a bf16 [Mp x N] matrix into fp32 db[N] (one block per column)
__global__ void colsum_kernel(const __nv_bfloat16 *__restrict__ Dt, int Mp, float *__restrict__ db) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < Mp; r += blockDim.x) s += __bfloat162float(Dt[(size_t)c * Mp + r]);
    __shared__ float sh[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) db[c] = s;
    }
}

// loss[0] = mean((y - t)^2) over real rows, also added into loss[1] (the
// epoch's running sum); dY (bf16, col 0, row-major and transposed) =
// 2 (y - t) / M.  One block.
__global__ void loss_kernel(const float *__restrict__ Y, const float *__restrict__ tgt, int M, int Mp,
                            __nv_bfloat16 *__restrict__ dY, __nv_bfloat16 *__restrict__ dYt, float *__restrict__ loss) {
    float s = 0.f;
    for (int r = threadIdx.x; r < Mp; r += blockDim.x) {
        float g = 0.f;
        if (r < M) {
            const float d = Y[(size_t)r * kOutPad] - tgt[r];
            s += d * d;
            g = 2.f * d / (float)M;
        }
        const __nv_bfloat16 b = __float2bfloat16(g);
        dY[(size_t)r * kOutPad] = b;
        dYt[r] = b;   // row 0 of dY^T
    }
    __shared__ float sh[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) {
            const float l = s / (float)(M > 0 ? M : 1);
            loss[0] = l;
            loss[1] += l;
        }
    }
}

// embedding gradient: demb[pid] += dX[r, 48..79]
__global__ void emb_grad_kernel(const float *__restrict__ dX, int ldx, const int32_t *__restrict__ pids, int M,
                                int n_ids, float *__restrict__ demb) {
    const int64_t n = (int64_t)M * kEmb;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / kEmb), c = (int)(i % kEmb);
        int p = pids[r];
        p = p < 0 ? 0 : (p > n_ids ? n_ids : p);
        atomicAdd(&demb[(size_t)p * kEmb + c], dX[(size_t)r * ldx + kIn + c]);
    }
}

// Adam over fp32 master weights; g, m, v, w all of length n.  The bias
// corrections (1 - b1^t, 1 - b2^t) of this step are cbias[*bidx], so that a
// captured step reads the current ones when it is replayed.
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                            const float2 *__restrict__ cbias, const int *__restrict__ bidx) {
    const float2 c = cbias[*bidx];
    const float c1 = c.x, c2 = c.y;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Batch *bidx of an epoch: rows order[*bidx * batch + i], i < M, of the
// device-resident samples into the step's input buffers.
__global__ void gather_batch_kernel(const float *__restrict__ all_feats, const int32_t *__restrict__ all_pids,
                                    const float *__restrict__ all_tgt, const int64_t *__restrict__ order,
                                    const int *__restrict__ bidx, int batch, int M, float *__restrict__ feats,
                                    int32_t *__restrict__ pids, float *__restrict__ tgt) {
    const int64_t b0 = (int64_t)(*bidx) * batch;
    const int64_t n = (int64_t)M * kIn;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / kIn), c = (int)(i % kIn);
        const int64_t j = order[b0 + r];
        feats[i] = all_feats[j * kIn + c];
        if (c == 0) {
            pids[r] = all_pids[j];
            tgt[r] = all_tgt[j];
        }
    }
}

// the next batch of the epoch
__global__ void bump_kernel(int *bidx) { ++*bidx; }

// bf16 copies of a weight matrix W [rows x cols] (fp32): row-major into Wb
// (ld = ldb, zero padded) and transposed into Wt (ld = ldt)
__global__ void weight_copy_kernel(const float *__restrict__ W, int rows, int cols, __nv_bfloat16 *__restrict__ Wb,
                                   int ldb, int rows_pad, __nv_bfloat16 *__restrict__ Wt, int ldt, int cols_pad) {
    const int64_t n = (int64_t)rows_pad * ldb;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / ldb), c = (int)(i % ldb);
        const float v = (r < rows && c < cols) ? W[(size_t)r * cols + c] : 0.f;
        Wb[i] = __float2bfloat16(v);
        if (c < cols_pad && r < ldt) Wt[(size_t)c * ldt + r] = __float2bfloat16(v);
    }
}

}  // namespace mlp
}  // namespace wk

using namespace wk;
using namespace wk::mlp;

struct wk_mlp {
    wk_ctx *ctx = nullptr;
    int n_ids = 0;
    int trusted = 1;             // cleared by wk_mlp_validate when held-out q-error exceeds its bound
    int cap_m = 0;               // padded batch capacity
    // fp32 master parameters, gradients, Adam moments (one contiguous block)
    float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
    int64_t n_params = 0;
    // views into params/grads
    int64_t off_w[4] = {}, off_b[4] = {}, off_emb = 0;
    // bf16 weights (row-major, padded) and transposes
    __nv_bfloat16 *wb[4] = {}, *wt[4] = {};
    // activations (capacity cap_m)
    // dz / dzt: two buffers, the layer whose weight gradient is taken and the one below it
    __nv_bfloat16 *x0 = nullptr, *x0t = nullptr, *h[3] = {}, *ht[3] = {}, *dz[2] = {}, *dzt[2] = {}, *dy = nullptr,
                  *dyt = nullptr;
    float *z[4] = {}, *dx = nullptr, *feats = nullptr, *tgt = nullptr, *loss = nullptr;
    int32_t *pids = nullptr;
    int *bidx = nullptr;         // the batch of the epoch a training step takes
    float2 *cbias = nullptr;     // Adam bias corrections of an epoch's steps
    int64_t cbias_cap = 0;
    int64_t step = 0;
    int64_t kernels = 0;
    int *d_err = nullptr;        // device flag of the tensor-core GEMM (bit 2: a wait ran out,
                                 // bit 3: work left in flight, TMEM kept)
    int *h_err = nullptr;        // pinned mirror
    int status = 0;              // a host-side GEMM failure since the last check
    int sms = 152;               // multiprocessors of the device (GEMM tile width choice)
    bool broken = false;         // a GEMM left work in flight: no further GEMM is launched
};

namespace {

const int kRows[4] = {kH, kH, kH, 1};        // output dim of each layer
const int kCols[4] = {kX, kH, kH, kH};       // input dim of each layer
const int kRowsPad[4] = {kH, kH, kH, kOutPad};

inline int pad64(int x) { return (x + 63) / 64 * 64; }
unsigned int nblk(int64_t n) { int64_t b = (n + 255) / 256; return (unsigned int)(b > 2048 ? 2048 : (b < 1 ? 1 : b)); }

void refresh_bf16(wk_mlp *m, cudaStream_t s) {
    for (int l = 0; l < 4; ++l) {
        // W^T of layer l is [cols x rows_pad]: the dX product takes it as B
        // with N = cols (layer 0 pads 80 -> 128; the extra rows stay zero)
        const int tcols = (l == 0) ? kXPadN : kH;
        weight_copy_kernel<<<nblk((int64_t)kRowsPad[l] * kCols[l]), 256, 0, s>>>(
            m->params + m->off_w[l], kRows[l], kCols[l], m->wb[l], kCols[l], kRowsPad[l], m->wt[l], kRowsPad[l], tcols);
    }
    m->kernels += 4;
}

// C = A . B^T (+ bias) on the tensor cores (wk_tc_gemm.cuh), with the
// epilogue EPI; N is a multiple of 64.  The tile width is the widest that still
// gives a full wave of CTAs, else 32: these products are small, and more CTAs
// means more copies and products in flight and more warps for the epilogue.
template <int EPI = tc::kEpiStore>
void gemm(wk_mlp *m, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, float *C, int ldc, int M, int N,
          int K, const float *bias, cudaStream_t s, const tc::EpiArgs &ea = tc::EpiArgs()) {
    if (m->broken) {
        if (!m->status)
            m->status = set_error(WK_EDEVICE, "estimator: an earlier tensor-core GEMM left work in flight; "
                                              "destroy the estimator");
        return;
    }
    if (M <= 0 || K <= 0 || N <= 0 || N % 64 || ldc % 4 || ((uintptr_t)C & 15u) || ((uintptr_t)bias & 15u) ||
        (EPI != tc::kEpiStore && (((uintptr_t)ea.h & 15u) || ea.ldh % 8 || !ea.ht || ea.m_store > M)) ||
        (EPI == tc::kEpiGeluBwd && (((uintptr_t)ea.z & 15u) || ea.ldz % 4 || !ea.colsum))) {
        if (!m->status) m->status = set_error(WK_EINVAL, "estimator GEMM: shape or alignment (M %d, N %d, K %d)", M, N, K);
        return;
    }
    const int mt = (M + tc::kTM - 1) / tc::kTM;
    const int bn = (N % 256 == 0 && mt * (N / 256) >= m->sms)   ? 256
                   : (N % 128 == 0 && mt * (N / 128) >= m->sms) ? 128
                   : (mt * (N / 64) >= m->sms)                  ? 64
                                                                : 32;
    CUtensorMap ta, tb;
    if (!tc::make_map(&ta, A, (uint64_t)M, (uint64_t)K, (uint64_t)lda, tc::kTM) ||
        !tc::make_map(&tb, B, (uint64_t)N, (uint64_t)K, (uint64_t)ldb, (uint32_t)bn)) {
        if (!m->status) m->status = set_error(WK_EDEVICE, "estimator GEMM: tensor map (M %d, N %d, K %d)", M, N, K);
        return;
    }
    const dim3 grid((unsigned)mt, (unsigned)(N / bn));
    switch (bn) {
        case 32:
            tc::gemm_tc_kernel<32, EPI><<<grid, tc::kThreads, tc::smem_bytes(32), s>>>(ta, tb, C, ldc, M, K, bias,
                                                                                       m->d_err, ea);
            break;
        case 64:
            tc::gemm_tc_kernel<64, EPI><<<grid, tc::kThreads, tc::smem_bytes(64), s>>>(ta, tb, C, ldc, M, K, bias,
                                                                                       m->d_err, ea);
            break;
        case 128:
            tc::gemm_tc_kernel<128, EPI><<<grid, tc::kThreads, tc::smem_bytes(128), s>>>(ta, tb, C, ldc, M, K, bias,
                                                                                         m->d_err, ea);
            break;
        default:
            tc::gemm_tc_kernel<256, EPI><<<grid, tc::kThreads, tc::smem_bytes(256), s>>>(ta, tb, C, ldc, M, K, bias,
                                                                                         m->d_err, ea);
            break;
    }
    m->kernels++;
}

// the epilogue operands of a hidden layer's activation: h / ht written for
// rows below Mp, values for rows below M
tc::EpiArgs act_args(int M, int Mp, __nv_bfloat16 *h, __nv_bfloat16 *ht, const float *z = nullptr,
                     float *colsum = nullptr) {
    tc::EpiArgs ea;
    ea.m_real = M;
    ea.m_store = Mp;
    ea.h = h;
    ea.ldh = kH;
    ea.ht = ht;
    ea.ldt = Mp;
    ea.z = z;
    ea.ldz = kH;
    ea.colsum = colsum;
    return ea;
}

template <int BN, int EPI>
bool set_gemm_smem() {
    return cudaFuncSetAttribute(tc::gemm_tc_kernel<BN, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tc::smem_bytes(BN)) == cudaSuccess;
}

template <int EPI>
bool set_gemm_smem_all() {
    return set_gemm_smem<32, EPI>() && set_gemm_smem<64, EPI>() && set_gemm_smem<128, EPI>() &&
           set_gemm_smem<256, EPI>();
}

// the status of the work queued since the last check: a host-side failure, a
// launch error, or a tensor-core wait that ran out (bit 2 of the device flag)
int check_status(wk_mlp *m, cudaStream_t s, const char *what) {
    int st = m->status;
    m->status = WK_OK;
    if (st) return st;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->h_err, m->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (*m->h_err) {
        const int f = *m->h_err;
        *m->h_err = 0;
        cudaMemsetAsync(m->d_err, 0, sizeof(int), s);
        if (f & 8) {
            // copies or products may still be in flight and their CTA kept its
            // TMEM: the estimator launches no further GEMM
            m->broken = true;
            return set_error(WK_EDEVICE, "%s: a tensor-core GEMM wait ran out with work in flight; "
                                         "destroy the estimator", what);
        }
        return set_error(WK_ETIMEDOUT, "%s: a tensor-core GEMM wait ran out", what);
    }
    return WK_OK;
}

// forward over M rows already uploaded (feats, pids); Y in z[3] col 0
void forward(wk_mlp *m, int M, cudaStream_t s) {
    const int Mp = pad64(M);
    build_input_kernel<<<nblk((int64_t)Mp * kX), 256, 0, s>>>(m->feats, m->pids, M, Mp, m->params + m->off_emb,
                                                              m->n_ids, m->x0, m->x0t);
    const __nv_bfloat16 *in = m->x0;
    int kin = kX;
    for (int l = 0; l < 3; ++l) {
        // Z_l = X W_l^T + b_l, and H_l = GELU(Z_l) from the epilogue
        gemm<tc::kEpiGeluFwd>(m, in, kin, m->wb[l], kin, m->z[l], kH, Mp, kH, kin, m->params + m->off_b[l], s,
                              act_args(M, Mp, m->h[l], m->ht[l]));
        in = m->h[l];
        kin = kH;
    }
    gemm(m, in, kH, m->wb[3], kH, m->z[3], kOutPad, Mp, kOutPad, kH, nullptr, s);
    // output bias (layer 4 has one real output): added in the loss / predict read
    m->kernels += 1;
}

// loss + backward + Adam on M rows (targets uploaded)
void backward_step(wk_mlp *m, int M, float lr, bool update, cudaStream_t s) {
    const int Mp = pad64(M);
    float *g = m->grads;
    cudaMemsetAsync(g, 0, sizeof(float) * (size_t)m->n_params, s);
    // dY: y includes the output bias
    loss_kernel<<<1, 1024, 0, s>>>(m->z[3], m->tgt, M, Mp, m->dy, m->dyt, m->loss);
    // layer 4: dW4 = dY^T . H3 (B = H3^T [256 x Mp]); db4 = sum dY; dZ3 = (dY . W4) * GELU'(Z3)
    // (B = W4^T [256 x 64]) with db3 from the same epilogue
    int cur = 0;
    {
        float *dw4 = g + m->off_w[3];   // [1 x 256] real, GEMM writes [64 x 256]
        gemm(m, m->dyt, Mp, m->ht[2], Mp, m->dx /*scratch [64 x 256]*/, kH, kOutPad, kH, Mp, nullptr, s);
        cudaMemcpyAsync(dw4, m->dx, sizeof(float) * kH, cudaMemcpyDeviceToDevice, s);   // row 0
        colsum_kernel<<<1, 256, 0, s>>>(m->dyt, Mp, g + m->off_b[3]);
        gemm<tc::kEpiGeluBwd>(m, m->dy, kOutPad, m->wt[3], kOutPad, nullptr, kH, Mp, kH, kOutPad, nullptr, s,
                              act_args(M, Mp, m->dz[cur], m->dzt[cur], m->z[2], g + m->off_b[2]));
    }
    for (int l = 2; l >= 0; --l) {
        // dZ_l is in dz[cur] / dzt[cur], db_l already summed
        const __nv_bfloat16 *inT = (l == 0) ? m->x0t : m->ht[l - 1];
        const int kin = (l == 0) ? kX : kH;
        // dW_l [256 x kin] = dZ^T [256 x Mp] . (X^T [kin x Mp])^T ; N = kin must be a multiple of 64
        if (kin % 64 == 0) {
            gemm(m, m->dzt[cur], Mp, inT, Mp, g + m->off_w[l], kin, kH, kin, Mp, nullptr, s);
        } else {
            // layer 0: kin = 80 -> compute into scratch [256 x 128] then copy the first 80 columns
            gemm(m, m->dzt[cur], Mp, inT, Mp, m->dx, kXPadN, kH, kXPadN, Mp, nullptr, s);
            cudaMemcpy2DAsync(g + m->off_w[0], sizeof(float) * kX, m->dx, sizeof(float) * kXPadN, sizeof(float) * kX,
                              kH, cudaMemcpyDeviceToDevice, s);
        }
        // dZ_{l-1} = (dZ_l . W_l) * GELU'(Z_{l-1}) (B = W_l^T [256 x 256]), with db_{l-1};
        // layer 0: dX = dZ_0 . W_0 (B = W_0^T [128 x 256]) for the embedding gradient
        if (l > 0) {
            gemm<tc::kEpiGeluBwd>(m, m->dz[cur], kH, m->wt[l], kH, nullptr, kH, Mp, kH, kH, nullptr, s,
                                  act_args(M, Mp, m->dz[1 - cur], m->dzt[1 - cur], m->z[l - 1], g + m->off_b[l - 1]));
            cur = 1 - cur;
        } else {
            gemm(m, m->dz[cur], kH, m->wt[0], kH, m->dx, kXPadN, Mp, kXPadN, kH, nullptr, s);
        }
    }
    emb_grad_kernel<<<nblk((int64_t)M * kEmb), 256, 0, s>>>(m->dx, kXPadN, m->pids, M, m->n_ids, g + m->off_emb);
    m->kernels += 3;
    if (update) {
        adam_kernel<<<nblk(m->n_params), 256, 0, s>>>(m->params, g, m->m1, m->m2, m->n_params, lr, kB1, kB2, 1e-8f,
                                                      m->cbias, m->bidx);
        refresh_bf16(m, s);
        m->kernels++;
    }
}

__global__ void add_bias_read_kernel(const float *Y, const float *b4, int M, float *out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < M; r += gridDim.x * blockDim.x) out[r] = Y[(size_t)r * kOutPad] + b4[0];
}

// add the output bias to column 0 of Y in place (so loss and predict see y = H3 . w4 + b4)
__global__ void add_out_bias_kernel(float *Y, const float *b4, int M) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < M; r += gridDim.x * blockDim.x) Y[(size_t)r * kOutPad] += b4[0];
}

int upload(wk_mlp *m, const float *feats, const int32_t *pids, const float *tgt, int M, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(m->feats, feats, sizeof(float) * (size_t)M * kIn, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->pids, pids, sizeof(int32_t) * (size_t)M, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && tgt) e = cudaMemcpyAsync(m->tgt, tgt, sizeof(float) * (size_t)M, cudaMemcpyHostToDevice, s);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "mlp upload");
}

void free_mlp(wk_mlp *m) {
    if (m->ctx && m->ctx->device >= 0) cudaSetDevice(m->ctx->device);
    cudaFree(m->params);
    cudaFree(m->grads);
    cudaFree(m->m1);
    cudaFree(m->m2);
    for (int l = 0; l < 4; ++l) { cudaFree(m->wb[l]); cudaFree(m->wt[l]); cudaFree(m->z[l]); }
    for (int l = 0; l < 3; ++l) { cudaFree(m->h[l]); cudaFree(m->ht[l]); }
    cudaFree(m->x0); cudaFree(m->x0t); cudaFree(m->dy); cudaFree(m->dyt);
    for (int i = 0; i < 2; ++i) { cudaFree(m->dz[i]); cudaFree(m->dzt[i]); }
    cudaFree(m->dx); cudaFree(m->feats); cudaFree(m->tgt); cudaFree(m->loss); cudaFree(m->pids);
    cudaFree(m->d_err);
    cudaFree(m->bidx);
    cudaFree(m->cbias);
    if (m->h_err) cudaFreeHost(m->h_err);
    delete m;
}

}  // namespace

extern "C" int wk_mlp_create(wk_ctx *ctx, int32_t n_ids, int32_t max_batch, uint64_t seed, wk_mlp **out) {
    if (!ctx || !out || n_ids < 1 || max_batch < 1 || max_batch > (1 << 20))
        return set_error(WK_EINVAL, "wk_mlp_create: bad arguments");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_mlp_create: host-only context");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    wk_mlp *m = new wk_mlp();
    m->ctx = ctx;
    m->n_ids = n_ids;
    m->cap_m = pad64(max_batch);
    cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int64_t at = 0;
    for (int l = 0; l < 4; ++l) { m->off_w[l] = at; at += (int64_t)kRows[l] * kCols[l]; }
    for (int l = 0; l < 4; ++l) { m->off_b[l] = at; at += kRowsPad[l]; }
    m->off_emb = at;
    at += (int64_t)(n_ids + 1) * kEmb;
    m->n_params = at;
    const size_t P = sizeof(float) * (size_t)at, Mp = (size_t)m->cap_m;
    bool ok = cudaMalloc(&m->params, P) == cudaSuccess && cudaMalloc(&m->grads, P) == cudaSuccess &&
              cudaMalloc(&m->m1, P) == cudaSuccess && cudaMalloc(&m->m2, P) == cudaSuccess;
    for (int l = 0; ok && l < 4; ++l) {
        const int tcols = (l == 0) ? kXPadN : kH;
        ok = cudaMalloc(&m->wb[l], 2 * (size_t)kRowsPad[l] * kCols[l]) == cudaSuccess &&
             cudaMalloc(&m->wt[l], 2 * (size_t)tcols * kRowsPad[l]) == cudaSuccess &&
             cudaMalloc(&m->z[l], 4 * Mp * (size_t)(l < 3 ? kH : kOutPad)) == cudaSuccess;
    }
    for (int l = 0; ok && l < 3; ++l)
        ok = cudaMalloc(&m->h[l], 2 * Mp * kH) == cudaSuccess && cudaMalloc(&m->ht[l], 2 * Mp * kH) == cudaSuccess;
    // X0^T has kXPadN rows: the layer-0 weight-gradient product pads N = 80 to 128 and reads rows 80..127 (zero)
    ok = ok && cudaMalloc(&m->x0, 2 * Mp * kX) == cudaSuccess && cudaMalloc(&m->x0t, 2 * Mp * kXPadN) == cudaSuccess &&
         cudaMalloc(&m->dz[0], 2 * Mp * kH) == cudaSuccess && cudaMalloc(&m->dzt[0], 2 * Mp * kH) == cudaSuccess &&
         cudaMalloc(&m->dz[1], 2 * Mp * kH) == cudaSuccess && cudaMalloc(&m->dzt[1], 2 * Mp * kH) == cudaSuccess &&
         cudaMalloc(&m->dy, 2 * Mp * kOutPad) == cudaSuccess && cudaMalloc(&m->dyt, 2 * Mp * kOutPad) == cudaSuccess &&
         cudaMalloc(&m->dx, 4 * std::max(Mp * (size_t)kXPadN, (size_t)kH * kXPadN)) == cudaSuccess &&
         cudaMalloc(&m->feats, 4 * Mp * kIn) == cudaSuccess && cudaMalloc(&m->tgt, 4 * Mp) == cudaSuccess &&
         cudaMalloc(&m->loss, 16) == cudaSuccess && cudaMalloc(&m->pids, 4 * Mp) == cudaSuccess &&
         cudaMalloc(&m->d_err, sizeof(int)) == cudaSuccess && cudaMalloc(&m->bidx, sizeof(int)) == cudaSuccess &&
         cudaHostAlloc((void **)&m->h_err, sizeof(int), 0) == cudaSuccess &&
         set_gemm_smem_all<tc::kEpiStore>() && set_gemm_smem_all<tc::kEpiGeluFwd>() &&
         set_gemm_smem_all<tc::kEpiGeluBwd>();
    if (!ok) {
        cudaGetLastError();
        free_mlp(m);
        return set_error(WK_ENOMEM, "wk_mlp_create: allocation failed");
    }
    // He-style initialisation (uniform with the fan-in bound), zero biases, small embeddings
    std::vector<float> h((size_t)at, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < 4; ++l) {
        const float bound = std::sqrt(6.f / (float)kCols[l]) * (l == 3 ? 0.5f : 1.f);
        std::uniform_real_distribution<float> U(-bound, bound);
        for (int64_t i = 0; i < (int64_t)kRows[l] * kCols[l]; ++i) h[(size_t)(m->off_w[l] + i)] = U(rng);
    }
    std::normal_distribution<float> Nrm(0.f, 0.1f);
    for (int64_t i = 0; i < (int64_t)(n_ids + 1) * kEmb; ++i) h[(size_t)(m->off_emb + i)] = Nrm(rng);
    cudaStream_t s = ctx->stream;
    e = cudaMemcpyAsync(m->params, h.data(), P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->m1, 0, P, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->m2, 0, P, s);
    for (int l = 0; e == cudaSuccess && l < 4; ++l) {
        const int tcols = (l == 0) ? kXPadN : kH;
        e = cudaMemsetAsync(m->wt[l], 0, 2 * (size_t)tcols * kRowsPad[l], s);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(m->x0t, 0, 2 * Mp * kXPadN, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->dy, 0, 2 * Mp * kOutPad, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->dyt, 0, 2 * Mp * kOutPad, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_err, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->bidx, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, 16, s);
    if (m->h_err) *m->h_err = 0;
    if (e != cudaSuccess) { int r = cuda_fail(e, "wk_mlp_create init"); free_mlp(m); return r; }
    refresh_bf16(m, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { int r = cuda_fail(e, "wk_mlp_create sync"); free_mlp(m); return r; }
    *out = m;
    return WK_OK;
}

extern "C" int wk_mlp_destroy(wk_mlp *m) {
    if (m) free_mlp(m);
    return WK_OK;
}

extern "C" int64_t wk_mlp_num_params(wk_mlp *m) { return m ? m->n_params : 0; }

// parameter block layout: W1 [256x80], W2, W3 [256x256], W4 [1x256], b1, b2, b3 [256], b4 [64, first used], emb [(n_ids+1) x 32]
extern "C" int wk_mlp_get_params(wk_mlp *m, float *host, int64_t n) {
    if (!m || !host || n < m->n_params) return set_error(WK_EINVAL, "wk_mlp_get_params");
    cudaError_t e = cudaMemcpy(host, m->params, sizeof(float) * (size_t)m->n_params, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "wk_mlp_get_params");
}

extern "C" int wk_mlp_set_params(wk_mlp *m, const float *host, int64_t n) {
    if (!m || !host || n < m->n_params) return set_error(WK_EINVAL, "wk_mlp_set_params");
    cudaSetDevice(m->ctx->device);
    cudaError_t e = cudaMemcpy(m->params, host, sizeof(float) * (size_t)m->n_params, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "wk_mlp_set_params");
    refresh_bf16(m, m->ctx->stream);
    e = cudaStreamSynchronize(m->ctx->stream);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "wk_mlp_set_params sync");
}

// One forward + backward on rows 0..M-1 without an update: loss and the
// gradients of every parameter (same layout as the parameters).
extern "C" int wk_mlp_gradients(wk_mlp *m, const float *feats, const int32_t *pids, const float *tgt, int32_t M,
                                float *grads_host, float *loss_host) {
    if (!m || !feats || !pids || !tgt || M < 1 || M > m->cap_m) return set_error(WK_EINVAL, "wk_mlp_gradients");
    cudaSetDevice(m->ctx->device);
    cudaStream_t s = m->ctx->stream;
    int st = upload(m, feats, pids, tgt, M, s);
    if (st) return st;
    forward(m, M, s);
    add_out_bias_kernel<<<nblk(M), 256, 0, s>>>(m->z[3], m->params + m->off_b[3], M);
    backward_step(m, M, 0.f, false, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && grads_host)
        e = cudaMemcpyAsync(grads_host, m->grads, sizeof(float) * (size_t)m->n_params, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && loss_host) e = cudaMemcpyAsync(loss_host, m->loss, 4, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "wk_mlp_gradients");
    return check_status(m, s, "wk_mlp_gradients");
}

// Mini-batch training: `epochs` passes over n samples in batches of `batch`
// (sample order shuffled with `seed`), Adam with learning rate lr.  Returns
// the mean loss of the last epoch.
//
// The samples are uploaded once and stay on the device; every step gathers
// its batch there by the epoch's order.  A step of a full batch is the same
// launch sequence every time (its batch index and Adam bias corrections are
// read from device memory), so the second full batch is captured as a CUDA
// graph and every later one replays it: one launch instead of about forty.
// A shorter last batch runs as plain launches.  The host reads the device
// once per epoch (the loss sum and the GEMM status).
extern "C" int wk_mlp_train(wk_mlp *m, const float *feats, const int32_t *pids, const float *tgt, int64_t n,
                            int32_t epochs, int32_t batch, float lr, uint64_t seed, float *last_loss) {
    if (!m || !feats || !pids || !tgt || n < 1 || epochs < 1 || batch < 1 || batch > m->cap_m)
        return set_error(WK_EINVAL, "wk_mlp_train: bad arguments");
    cudaError_t e = cudaSetDevice(m->ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    cudaStream_t s = m->ctx->stream;
    const int64_t nb = (n + batch - 1) / batch, nfull = n / batch;
    const int tail = (int)(n - nfull * batch);
    DevBuf d_feats, d_pids, d_tgt, d_order;
    int st;
    if ((st = d_feats.reserve(sizeof(float) * (size_t)n * kIn)) || (st = d_pids.reserve(sizeof(int32_t) * (size_t)n)) ||
        (st = d_tgt.reserve(sizeof(float) * (size_t)n)) || (st = d_order.reserve(sizeof(int64_t) * (size_t)n)))
        return st;
    if (nb > m->cbias_cap) {
        cudaFree(m->cbias);
        m->cbias = nullptr;
        m->cbias_cap = 0;
        if ((e = cudaMalloc(&m->cbias, sizeof(float2) * (size_t)nb)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(WK_ENOMEM, "wk_mlp_train: bias-correction table");
        }
        m->cbias_cap = nb;
    }
    if ((e = cudaMemcpyAsync(d_feats.ptr, feats, sizeof(float) * (size_t)n * kIn, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(d_pids.ptr, pids, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(d_tgt.ptr, tgt, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, s)))
        return cuda_fail(e, "wk_mlp_train upload");
    std::vector<int64_t> order((size_t)n);
    for (int64_t i = 0; i < n; ++i) order[(size_t)i] = i;
    std::vector<float2> cb((size_t)nb);
    std::mt19937_64 rng(seed);
    float *h_loss = nullptr;
    if (cudaHostAlloc((void **)&h_loss, 8, 0) != cudaSuccess) return set_error(WK_ENOMEM, "wk_mlp_train: pinned");
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graph_kernels = 0;
    auto one_step = [&](int M) {
        gather_batch_kernel<<<nblk((int64_t)M * kIn), 256, 0, s>>>(d_feats.as<float>(), d_pids.as<int32_t>(),
                                                                   d_tgt.as<float>(), d_order.as<int64_t>(), m->bidx,
                                                                   batch, M, m->feats, m->pids, m->tgt);
        forward(m, M, s);
        add_out_bias_kernel<<<nblk(M), 256, 0, s>>>(m->z[3], m->params + m->off_b[3], M);
        backward_step(m, M, lr, true, s);
        bump_kernel<<<1, 1, 0, s>>>(m->bidx);
        m->kernels += 4;   // gather, output bias, Adam, bump
    };
    auto finish = [&](int rc) {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamSynchronize(s);   // the pinned loss and the device samples may still be in use
        cudaFreeHost(h_loss);
        m->ctx->launches += m->kernels;
        m->kernels = 0;
        return rc;
    };
    double ep_loss = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        // Adam step t = step + k + 1 for batch k of this epoch
        for (int64_t k = 0; k < nb; ++k) {
            const float t = (float)(m->step + k + 1);
            cb[(size_t)k] = make_float2(1.f - std::pow(kB1, t), 1.f - std::pow(kB2, t));
        }
        if ((e = cudaMemcpyAsync(d_order.ptr, order.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(m->cbias, cb.data(), sizeof(float2) * (size_t)nb, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemsetAsync(m->bidx, 0, sizeof(int), s)) || (e = cudaMemsetAsync(m->loss + 1, 0, sizeof(float), s)))
            return finish(cuda_fail(e, "wk_mlp_train epoch"));
        for (int64_t k = 0; k < nfull; ++k) {
            if (exec) {
                if ((e = cudaGraphLaunch(exec, s)) != cudaSuccess) return finish(cuda_fail(e, "wk_mlp_train replay"));
                m->kernels += graph_kernels;
            } else if (k == 0 && ep == 0) {
                one_step(batch);
            } else {
                const int64_t k0 = m->kernels;
                if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                    return finish(cuda_fail(e, "wk_mlp_train capture"));
                one_step(batch);
                e = cudaStreamEndCapture(s, &graph);
                graph_kernels = m->kernels - k0;
                m->kernels = k0;
                if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
                if (e != cudaSuccess) return finish(cuda_fail(e, "wk_mlp_train graph"));
                if ((e = cudaGraphLaunch(exec, s)) != cudaSuccess) return finish(cuda_fail(e, "wk_mlp_train replay"));
                m->kernels += graph_kernels;
            }
        }
        if (tail) one_step(tail);
        m->step += nb;
        if ((e = cudaMemcpyAsync(h_loss, m->loss, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return finish(cuda_fail(e, "wk_mlp_train loss"));
        if ((st = check_status(m, s, "wk_mlp_train"))) return finish(st);
        ep_loss = (double)h_loss[1] / (double)nb;
    }
    if (last_loss) *last_loss = (float)ep_loss;
    return finish(WK_OK);
}

// Predictions (log(1 + rows)) for n samples, in chunks of the batch capacity.
extern "C" int wk_mlp_predict(wk_mlp *m, const float *feats, const int32_t *pids, int64_t n, float *out) {
    if (!m || (n > 0 && (!feats || !pids || !out)) || n < 0) return set_error(WK_EINVAL, "wk_mlp_predict");
    cudaSetDevice(m->ctx->device);
    cudaStream_t s = m->ctx->stream;
    for (int64_t b0 = 0; b0 < n; b0 += m->cap_m) {
        const int M = (int)std::min<int64_t>(m->cap_m, n - b0);
        int st = upload(m, feats + b0 * kIn, pids + b0, nullptr, M, s);
        if (st) return st;
        forward(m, M, s);
        add_bias_read_kernel<<<nblk(M), 256, 0, s>>>(m->z[3], m->params + m->off_b[3], M, m->tgt);
        cudaError_t e = cudaMemcpyAsync(out + b0, m->tgt, sizeof(float) * (size_t)M, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(e, "wk_mlp_predict");
        if ((st = check_status(m, s, "wk_mlp_predict"))) return st;
    }
    m->ctx->launches += m->kernels;
    m->kernels = 0;
    return WK_OK;
}

// Held-out check of the model: q-error of each sample is exp(|predicted -
// true|) in log(1 + rows) (the ratio of the larger to the smaller of rows + 1;
// a negative prediction counts as 0, as the planners clamp it).  The model is
// trusted while the 95th percentile stays within qerror_bound; an untrusted
// model makes the learned planners return the statistics plan.
extern "C" int wk_mlp_validate(wk_mlp *m, const float *feats, const int32_t *pids, const float *target, int64_t n,
                               double qerror_bound, double *p95_qerror, int32_t *trusted) {
    if (!m || n < 1 || !feats || !pids || !target || !(qerror_bound >= 1.0))
        return set_error(WK_EINVAL, "wk_mlp_validate: bad arguments");
    std::vector<float> pred((size_t)n);
    int st = wk_mlp_predict(m, feats, pids, n, pred.data());
    if (st) return st;
    std::vector<double> q((size_t)n);
    for (int64_t i = 0; i < n; ++i)
        q[(size_t)i] = std::exp(std::fabs((double)std::max(0.f, pred[(size_t)i]) - (double)target[(size_t)i]));
    const size_t k = (size_t)std::ceil(0.95 * (double)n) - 1;
    std::nth_element(q.begin(), q.begin() + (ptrdiff_t)k, q.end());
    const double p95 = q[k];
    m->trusted = p95 <= qerror_bound ? 1 : 0;
    if (p95_qerror) *p95_qerror = p95;
    if (trusted) *trusted = m->trusted;
    return WK_OK;
}

extern "C" int wk_mlp_is_trusted(wk_mlp *m) { return m ? m->trusted : 0; }
