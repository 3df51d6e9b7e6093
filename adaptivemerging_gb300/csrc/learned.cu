// learned.cu -- learned warm start for the batched solve.
//
// A small MLP (24 -> 64 -> 64 -> 3, GELU) maps per-contact features to the
// converged multipliers, expressed in velocity units (lambda_r * D_rr) so the
// mapping is insensitive to body mass.  Everything runs on the device:
//   * k_features  : the 24 features of every contact after warm start and
//                   solver setup (free contact velocity b, penetration / dt,
//                   normal, previous-frame impulse * D, persistence, mu,
//                   log-D ratios, mass split, contacts in the pair, ...);
//   * k_labels    : (lambda - lambda_warm) * D of the converged solve, the
//                   change from the previous-frame start (recorded for the
//                   contacts in scope of scenes that reached the target);
//   * training    : FP32 forward (k_fwd), backward as per-sample deltas
//                   (k_bwd_delta) then one thread per parameter and sample
//                   chunk for the weight gradients (k_bwd_grad), Adam
//                   (k_adam), MSE loss;
//   * inference   : BF16 weights on the tensor cores (mma.sync m16n8k16,
//                   FP32 accumulate); the 16 x 8 accumulator tiles of one
//                   layer are re-packed in registers as the A operand of the
//                   next, so activations never leave the warp;
//   * lambda_warm + prediction / D, projected (lambda_n >= 0,
//                   |lambda_t| <= mu lambda_n), becomes the start of the
//                   contacts in scope: fresh contacts only (scope 0, whose
//                   plain start is zero) or all contacts (scope 1).
// Features are standardised with the training set's mean and deviation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {

// parameter vector layout (floats)
static const int NIN = 24, NH = 64, NOUT = 3;
static const int OW1 = 0, OB1 = OW1 + NH * NIN, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
                 OB3 = OW3 + NOUT * NH, NPAR = OB3 + NOUT;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.3989422804014327f * expf(-0.5f * x * x);
}

// ---------------------------------------------------------------------------
// features / labels
__global__ void k_features(DBodies B, DContacts C, DPairs P, int nc, float dt, int fo, float fv, float* X) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int cap = C.cap;
    float f[NIN];
    double D[3];
    for (int r = 0; r < 3; r++) D[r] = C.bD[(3 + r) * cap + c];
    for (int r = 0; r < 3; r++) f[r] = (float)C.bD[r * cap + c];
    f[3] = (float)(C.cv[c] / dt);
    for (int k = 0; k < 3; k++) f[4 + k] = (float)C.J[(6 + k) * cap + c];   // jnb.v = normal
    for (int r = 0; r < 3; r++) f[7 + r] = (float)(C.lamw[r * cap + c] * D[r]);
    f[10] = C.fresh[c] ? 0.f : 1.f;
    float mu;
    if (fo) mu = fv;
    else {
        float f1 = (float)B.friction[C.b1[c]], f2 = (float)B.friction[C.b2[c]];
        if (f1 < 0.2f || f2 < 0.2f) mu = fminf(f1, f2);
        else if (f1 > 1.f || f2 > 1.f) mu = fmaxf(f1, f2);
        else mu = 0.5f * (f1 + f2);
    }
    f[11] = mu;
    f[12] = (float)log(D[0]);
    f[13] = (float)log(D[1] / D[0]);
    f[14] = (float)log(D[2] / D[0]);
    double m1 = B.minv[C.sb1[c]], m2 = B.minv[C.sb2[c]];
    f[15] = (float)(m1 / (m1 + m2 + 1e-30));
    f[16] = (float)P.count[C.pair[c]] * 0.125f;
    f[17] = (float)C.info[c] * 0.125f;
    double l0 = C.lamw[c];
    f[18] = (float)(C.lamw[cap + c] / (mu * l0 + 1e-12));
    f[19] = (float)(C.lamw[2 * cap + c] / (mu * l0 + 1e-12));
    f[20] = (float)(C.bD[c] + 0.5 * C.cv[c] / dt);
    f[21] = (float)C.cv[c];
    f[22] = (float)(C.bD[c] * D[0] > 0 ? 1.f : 0.f);
    f[23] = 1.f;
    for (int k = 0; k < NIN; k++) X[(size_t)c * NIN + k] = f[k];
}

// label: the converged impulse's change from the previous-frame start, in
// velocity units ((lambda - lambda_warm) * D); for a fresh contact the start
// is zero and the label is lambda * D
__global__ void k_labels(DContacts C, int nc, float* Y) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int cap = C.cap;
    for (int r = 0; r < 3; r++)
        Y[(size_t)c * NOUT + r] = (float)((C.lam[r * cap + c] - C.lamw[r * cap + c]) * C.bD[(3 + r) * cap + c]);
}

// keep flag: a contact in scope (fresh ones, or all) whose scene reached the
// residual target
__global__ void k_keep_converged(DContacts C, int nc, const int* sceneOf, const float* sceneRes, float tol, int all,
                                 int* keep) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    keep[c] = ((all || C.fresh[c]) && sceneRes[sceneOf[C.b1[c]]] <= tol) ? 1 : 0;
}

__global__ void k_append(const float* X, const float* Y, const int* keep, const int* pos, int nc, float* DX,
                         float* DY, int base, int cap) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc || !keep[c]) return;
    int d = base + pos[c];
    if (d >= cap) return;
    for (int k = 0; k < NIN; k++) DX[(size_t)d * NIN + k] = X[(size_t)c * NIN + k];
    for (int k = 0; k < NOUT; k++) DY[(size_t)d * NOUT + k] = Y[(size_t)c * NOUT + k];
}

// ---------------------------------------------------------------------------
// training (FP32)
__global__ void k_fwd(const float* __restrict__ X, const float* __restrict__ norm, const float* __restrict__ W,
                      const int* __restrict__ idx, int n, float* Z1, float* Z2, float* Yh) {
    __shared__ float w[NPAR];
    __shared__ float nm[2 * NIN];
    for (int k = threadIdx.x; k < NPAR; k += blockDim.x) w[k] = W[k];
    for (int k = threadIdx.x; k < 2 * NIN; k += blockDim.x) nm[k] = norm[k];
    __syncthreads();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int src = idx ? idx[s] : s;
    float x[NIN], a1[NH];
    for (int k = 0; k < NIN; k++) x[k] = (X[(size_t)src * NIN + k] - nm[k]) * nm[NIN + k];
    for (int o = 0; o < NH; o++) {
        float z = w[OB1 + o];
        for (int k = 0; k < NIN; k++) z = fmaf(w[OW1 + o * NIN + k], x[k], z);
        Z1[(size_t)s * NH + o] = z;
        a1[o] = gelu(z);
    }
    float y[NOUT];
    for (int q = 0; q < NOUT; q++) y[q] = w[OB3 + q];
    for (int o = 0; o < NH; o++) {
        float z = w[OB2 + o];
        for (int k = 0; k < NH; k++) z = fmaf(w[OW2 + o * NH + k], a1[k], z);
        Z2[(size_t)s * NH + o] = z;
        float a = gelu(z);
        for (int q = 0; q < NOUT; q++) y[q] = fmaf(w[OW3 + q * NH + o], a, y[q]);
    }
    for (int q = 0; q < NOUT; q++) Yh[(size_t)s * NOUT + q] = y[q];
}

// Backward in two kernels.  k_bwd_delta: one thread per sample computes the
// per-sample deltas (dy, dz2, dz1), the activations the weight gradients need,
// the normalised inputs and the MSE loss (mean over samples and outputs).
__global__ void k_bwd_delta(const float* __restrict__ X, const float* __restrict__ Yt,
                            const float* __restrict__ norm, const float* __restrict__ W, const int* __restrict__ idx,
                            int n, const float* __restrict__ Z1, const float* __restrict__ Z2,
                            const float* __restrict__ Yh, float* XN, float* A1, float* A2, float* D1, float* D2,
                            float* DY, float* loss) {
    __shared__ float w[NPAR];
    __shared__ float nm[2 * NIN];
    __shared__ float sl;
    for (int k = threadIdx.x; k < NPAR; k += blockDim.x) w[k] = W[k];
    for (int k = threadIdx.x; k < 2 * NIN; k += blockDim.x) nm[k] = norm[k];
    if (threadIdx.x == 0) sl = 0.f;
    __syncthreads();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) {
        int src = idx ? idx[s] : s;
        for (int k = 0; k < NIN; k++) XN[(size_t)s * NIN + k] = (X[(size_t)src * NIN + k] - nm[k]) * nm[NIN + k];
        float dy[NOUT], l = 0.f;
        const float scale = 2.f / (float)(n * NOUT);
        for (int q = 0; q < NOUT; q++) {
            float e = Yh[(size_t)s * NOUT + q] - Yt[(size_t)src * NOUT + q];
            l += e * e;
            dy[q] = scale * e;
            DY[(size_t)s * NOUT + q] = dy[q];
        }
        atomicAdd(&sl, l);
        float dz2[NH];
        for (int o = 0; o < NH; o++) {
            float z = Z2[(size_t)s * NH + o];
            A2[(size_t)s * NH + o] = gelu(z);
            float da = 0.f;
            for (int q = 0; q < NOUT; q++) da = fmaf(w[OW3 + q * NH + o], dy[q], da);
            dz2[o] = da * gelu_d(z);
            D2[(size_t)s * NH + o] = dz2[o];
        }
        for (int k = 0; k < NH; k++) {
            float z = Z1[(size_t)s * NH + k];
            A1[(size_t)s * NH + k] = gelu(z);
            float da = 0.f;
            for (int o = 0; o < NH; o++) da = fmaf(w[OW2 + o * NH + k], dz2[o], da);
            D1[(size_t)s * NH + k] = da * gelu_d(z);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(loss, sl / (float)(n * NOUT));
}

// k_bwd_grad: one thread per parameter and chunk of GCH samples sums that
// parameter's gradient over the chunk (deltas x activations, no atomics
// between samples) and adds it to G once.  Consecutive parameters read
// consecutive activations of a sample, so the loads coalesce.
static const int GCH = 128;
__global__ void k_bwd_grad(const float* __restrict__ XN, const float* __restrict__ A1, const float* __restrict__ A2,
                           const float* __restrict__ D1, const float* __restrict__ D2, const float* __restrict__ DY,
                           int n, float* G) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPAR) return;
    int s0 = blockIdx.y * GCH, s1 = min(n, s0 + GCH);
    float acc = 0.f;
    if (p < OB1) {
        int o = p / NIN, i = p % NIN;
        for (int s = s0; s < s1; s++) acc = fmaf(D1[(size_t)s * NH + o], XN[(size_t)s * NIN + i], acc);
    } else if (p < OW2) {
        int o = p - OB1;
        for (int s = s0; s < s1; s++) acc += D1[(size_t)s * NH + o];
    } else if (p < OB2) {
        int o = (p - OW2) / NH, k = (p - OW2) % NH;
        for (int s = s0; s < s1; s++) acc = fmaf(D2[(size_t)s * NH + o], A1[(size_t)s * NH + k], acc);
    } else if (p < OW3) {
        int o = p - OB2;
        for (int s = s0; s < s1; s++) acc += D2[(size_t)s * NH + o];
    } else if (p < OB3) {
        int q = (p - OW3) / NH, o = (p - OW3) % NH;
        for (int s = s0; s < s1; s++) acc = fmaf(DY[(size_t)s * NOUT + q], A2[(size_t)s * NH + o], acc);
    } else {
        int q = p - OB3;
        for (int s = s0; s < s1; s++) acc += DY[(size_t)s * NOUT + q];
    }
    atomicAdd(&G[p], acc);
}

__global__ void k_adam(float* W, const float* G, float* M, float* V, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float g = G[k];
    float m = b1 * M[k] + (1.f - b1) * g;
    float v = b2 * V[k] + (1.f - b2) * g * g;
    M[k] = m;
    V[k] = v;
    W[k] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
}

// ---------------------------------------------------------------------------
// inference: BF16 tensor cores.  One warp computes 16 contacts; the weights
// (transposed, BF16) sit in shared memory.
__device__ __forceinline__ unsigned pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

__device__ __forceinline__ void mma16816(float d[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// weights in shared memory as [n][k] BF16 pairs: layer l stores Wt[n][kpad]
static const int K1P = 32;   // 24 inputs padded to two k16 steps
__global__ void k_infer_bf16(const float* __restrict__ X, const float* __restrict__ norm,
                             const __nv_bfloat16* __restrict__ Wb, const float* __restrict__ bias, int n,
                             float* out) {
    // Wb layout: W1t [64][32], W2t [64][64], W3t [8][64]   (row n, k contiguous)
    __shared__ __align__(16) __nv_bfloat16 w1[NH * K1P];
    __shared__ __align__(16) __nv_bfloat16 w2[NH * NH];
    __shared__ __align__(16) __nv_bfloat16 w3[8 * NH];
    __shared__ float bs[NH + NH + 8];
    __shared__ float nm[2 * NIN];
    for (int k = threadIdx.x; k < NH * K1P; k += blockDim.x) w1[k] = Wb[k];
    for (int k = threadIdx.x; k < NH * NH; k += blockDim.x) w2[k] = Wb[NH * K1P + k];
    for (int k = threadIdx.x; k < 8 * NH; k += blockDim.x) w3[k] = Wb[NH * K1P + NH * NH + k];
    for (int k = threadIdx.x; k < NH + NH + 8; k += blockDim.x) bs[k] = bias[k];
    for (int k = threadIdx.x; k < 2 * NIN; k += blockDim.x) nm[k] = norm[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int row0 = warp * 16;
    if (row0 >= n) return;
    auto xin = [&](int row, int col) -> float {
        int r = row0 + row;
        if (r >= n || col >= NIN) return 0.f;
        return (X[(size_t)r * NIN + col] - nm[col]) * nm[NIN + col];
    };
    auto bfrag = [&](const __nv_bfloat16* w, int kp, int nt, int kk, unsigned b[2]) {
        const __nv_bfloat16* p = w + (nt * 8 + gid) * kp + kk * 16 + tig * 2;
        b[0] = *reinterpret_cast<const unsigned*>(p);
        b[1] = *reinterpret_cast<const unsigned*>(p + 8);
    };
    // layer 1: [16 x 32] x [32 x 64]
    float h[8][4];
    for (int nt = 0; nt < 8; nt++)
        for (int q = 0; q < 4; q++) h[nt][q] = 0.f;
    for (int kk = 0; kk < 2; kk++) {
        unsigned a[4];
        int c0 = kk * 16 + tig * 2;
        a[0] = pack2(xin(gid, c0), xin(gid, c0 + 1));
        a[1] = pack2(xin(gid + 8, c0), xin(gid + 8, c0 + 1));
        a[2] = pack2(xin(gid, c0 + 8), xin(gid, c0 + 9));
        a[3] = pack2(xin(gid + 8, c0 + 8), xin(gid + 8, c0 + 9));
        for (int nt = 0; nt < 8; nt++) {
            unsigned b[2];
            bfrag(w1, K1P, nt, kk, b);
            mma16816(h[nt], a, b);
        }
    }
    for (int nt = 0; nt < 8; nt++) {
        int col = nt * 8 + tig * 2;
        h[nt][0] = gelu(h[nt][0] + bs[col]);
        h[nt][1] = gelu(h[nt][1] + bs[col + 1]);
        h[nt][2] = gelu(h[nt][2] + bs[col]);
        h[nt][3] = gelu(h[nt][3] + bs[col + 1]);
    }
    // layer 2: accumulator tiles 2kk, 2kk+1 become the A operand of k-step kk
    float h2[8][4];
    for (int nt = 0; nt < 8; nt++)
        for (int q = 0; q < 4; q++) h2[nt][q] = 0.f;
    for (int kk = 0; kk < 4; kk++) {
        unsigned a[4] = {pack2(h[2 * kk][0], h[2 * kk][1]), pack2(h[2 * kk][2], h[2 * kk][3]),
                         pack2(h[2 * kk + 1][0], h[2 * kk + 1][1]), pack2(h[2 * kk + 1][2], h[2 * kk + 1][3])};
        for (int nt = 0; nt < 8; nt++) {
            unsigned b[2];
            bfrag(w2, NH, nt, kk, b);
            mma16816(h2[nt], a, b);
        }
    }
    for (int nt = 0; nt < 8; nt++) {
        int col = nt * 8 + tig * 2;
        h2[nt][0] = gelu(h2[nt][0] + bs[NH + col]);
        h2[nt][1] = gelu(h2[nt][1] + bs[NH + col + 1]);
        h2[nt][2] = gelu(h2[nt][2] + bs[NH + col]);
        h2[nt][3] = gelu(h2[nt][3] + bs[NH + col + 1]);
    }
    // layer 3: [16 x 64] x [64 x 8] (3 outputs used)
    float y[4] = {0.f, 0.f, 0.f, 0.f};
    for (int kk = 0; kk < 4; kk++) {
        unsigned a[4] = {pack2(h2[2 * kk][0], h2[2 * kk][1]), pack2(h2[2 * kk][2], h2[2 * kk][3]),
                         pack2(h2[2 * kk + 1][0], h2[2 * kk + 1][1]), pack2(h2[2 * kk + 1][2], h2[2 * kk + 1][3])};
        unsigned b[2];
        bfrag(w3, NH, 0, kk, b);
        mma16816(y, a, b);
    }
    int col = tig * 2;
    for (int half = 0; half < 2; half++) {
        int r = row0 + gid + 8 * half;
        if (r >= n) continue;
        for (int q = 0; q < 2; q++) {
            int o = col + q;
            if (o < NOUT) out[(size_t)r * NOUT + o] = y[2 * half + q] + bs[2 * NH + o];
        }
    }
}

// FP32 inference (reference path of the tests and the fallback when the
// tensor-core kernel is disabled)
__global__ void k_infer_f32(const float* X, const float* norm, const float* W, int n, float* out) {
    __shared__ float w[NPAR];
    __shared__ float nm[2 * NIN];
    for (int k = threadIdx.x; k < NPAR; k += blockDim.x) w[k] = W[k];
    for (int k = threadIdx.x; k < 2 * NIN; k += blockDim.x) nm[k] = norm[k];
    __syncthreads();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[NIN], a1[NH];
    for (int k = 0; k < NIN; k++) x[k] = (X[(size_t)s * NIN + k] - nm[k]) * nm[NIN + k];
    for (int o = 0; o < NH; o++) {
        float z = w[OB1 + o];
        for (int k = 0; k < NIN; k++) z = fmaf(w[OW1 + o * NIN + k], x[k], z);
        a1[o] = gelu(z);
    }
    float y[NOUT];
    for (int q = 0; q < NOUT; q++) y[q] = w[OB3 + q];
    for (int o = 0; o < NH; o++) {
        float z = w[OB2 + o];
        for (int k = 0; k < NH; k++) z = fmaf(w[OW2 + o * NH + k], a1[k], z);
        float a = gelu(z);
        for (int q = 0; q < NOUT; q++) y[q] = fmaf(w[OW3 + q * NH + o], a, y[q]);
    }
    for (int q = 0; q < NOUT; q++) out[(size_t)s * NOUT + q] = y[q];
}

// BF16 transposed weight images + bias vector for the inference kernel
__global__ void k_pack_bf16(const float* W, __nv_bfloat16* Wb, float* bias) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < NH * K1P) {
        int o = k / K1P, i = k % K1P;
        Wb[k] = __float2bfloat16(i < NIN ? W[OW1 + o * NIN + i] : 0.f);
    }
    if (k < NH * NH) Wb[NH * K1P + k] = __float2bfloat16(W[OW2 + k]);
    if (k < 8 * NH) {
        int o = k / NH, i = k % NH;
        Wb[NH * K1P + NH * NH + k] = __float2bfloat16(o < NOUT ? W[OW3 + o * NH + i] : 0.f);
    }
    if (k < NH) { bias[k] = W[OB1 + k]; bias[NH + k] = W[OB2 + k]; }
    if (k < 8) bias[2 * NH + k] = k < NOUT ? W[OB3 + k] : 0.f;
}

// learned start = previous-frame start + y / D, projected on the friction
// cone, packed (4 floats per contact, slot order) as the batched solver's start.  With
// scope 0 only fresh contacts (no previous-frame impulse) take it; the others
// keep the plain start, already the converged impulse of the last step.
__global__ void k_apply_prediction(DBodies B, DContacts C, int nc, const float* Yp, int fo, float fv, int all,
                                   const int* slotOf, const float* lamPlain, float* lamL) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int sl = slotOf[c];
    if (!all && !C.fresh[c]) {
        for (int r = 0; r < 4; r++) lamL[4 * sl + r] = lamPlain[4 * sl + r];
        return;
    }
    int cap = C.cap;
    double l[3];
    for (int r = 0; r < 3; r++)
        l[r] = C.lamw[r * cap + c] + (double)Yp[(size_t)c * NOUT + r] / C.bD[(3 + r) * cap + c];
    double mu;
    if (fo) mu = fv;
    else {
        double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
        if (f1 < 0.2 || f2 < 0.2) mu = fmin(f1, f2);
        else if (f1 > 1. || f2 > 1.) mu = fmax(f1, f2);
        else mu = (f1 + f2) / 2.;
    }
    l[0] = l[0] > 0 ? l[0] : 0.0;
    double lim = mu * l[0];
    for (int r = 1; r < 3; r++) l[r] = fmin(fmax(l[r], -lim), lim);
    for (int r = 0; r < 3; r++) lamL[4 * sl + r] = (float)l[r];
    lamL[4 * sl + 3] = (float)mu;   // the slot's fourth float carries mu for the sweep
}

// ---------------------------------------------------------------------------
// host side
int Ctx::learnedInit() {
    if (lW) return AM_OK;
    if (alloc(&lW, NPAR) || alloc(&lG, NPAR) || alloc(&lM, NPAR) || alloc(&lV, NPAR) || alloc(&lNorm, 2 * NIN) ||
        alloc(&lWb, NH * K1P + NH * NH + 8 * NH) || alloc(&lBias, 2 * NH + 8) || alloc(&lLoss, 1))
        return AM_E_CUDA;
    // He-style init from a fixed LCG (deterministic), zero biases, unit normalisation
    std::vector<float> w(NPAR, 0.f), nm(2 * NIN);
    unsigned st = 12345u;
    auto rnd = [&]() { st = st * 1664525u + 1013904223u; return ((st >> 8) & 0xFFFFFF) / 16777216.f * 2.f - 1.f; };
    for (int k = 0; k < NH * NIN; k++) w[OW1 + k] = rnd() * std::sqrt(6.f / NIN);
    for (int k = 0; k < NH * NH; k++) w[OW2 + k] = rnd() * std::sqrt(6.f / NH);
    for (int k = 0; k < NOUT * NH; k++) w[OW3 + k] = rnd() * std::sqrt(1.f / NH);
    for (int k = 0; k < NIN; k++) { nm[k] = 0.f; nm[NIN + k] = 1.f; }
    cudaMemcpyAsync(lW, w.data(), sizeof(float) * NPAR, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(lNorm, nm.data(), sizeof(float) * 2 * NIN, cudaMemcpyHostToDevice, stream);
    cudaMemsetAsync(lM, 0, sizeof(float) * NPAR, stream);
    cudaMemsetAsync(lV, 0, sizeof(float) * NPAR, stream);
    lAdamT = 0;
    return syncErr();
}

int Ctx::ensureFeat(int nc) {
    if (nc <= lFeatCap) return AM_OK;
    int cap = std::max(nc + nc / 2, 4096);
    if (alloc(&lX, (size_t)NIN * cap) || alloc(&lY, (size_t)NOUT * cap) || alloc(&lKeep, cap) || alloc(&lPos, cap))
        return AM_E_CUDA;
    lFeatCap = cap;
    return ensureScratch(cap + 1);
}

// features of the current contacts (after batchSolve's setup)
int Ctx::learnedFeatures(double dt) {
    int nc = nContacts;
    int r = ensureFeat(nc);
    if (r) return r;
    k_features<<<(nc + 127) / 128, 128, 0, stream>>>(B, C[cur], PR, nc, (float)dt, P.friction_override,
                                                     (float)P.friction, lX);
    AM_LAUNCHED(1);
    return AM_OK;
}

// record (features, converged lambda * D) of the scenes that reached the target
int Ctx::learnedRecord() {
    int nc = nContacts;
    if (!lCollect || nc <= 0) return AM_OK;
    k_labels<<<(nc + 127) / 128, 128, 0, stream>>>(C[cur], nc, lY);
    k_keep_converged<<<(nc + 127) / 128, 128, 0, stream>>>(C[cur], nc, sceneOfDev, bRes, (float)batchTol, lScope,
                                                           lKeep);
    AM_LAUNCHED(2);
    int* total = &dc->need_contacts;   // scratch counter
    launch_scan(lKeep, lPos, nc, SC, total, stream);
    int nkeep = 0;
    cudaMemcpyAsync(&nkeep, total, sizeof(int), cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    k_append<<<(nc + 127) / 128, 128, 0, stream>>>(lX, lY, lKeep, lPos, nc, lDX, lDY, lDn, lDcap);
    AM_LAUNCHED(1);
    lDn = std::min(lDcap, lDn + nkeep);
    return syncErr();
}

int Ctx::learnedPredict(bool tensorCores) {
    int nc = nContacts;
    if (nc <= 0) return AM_OK;
    if (tensorCores) {
        k_infer_bf16<<<(nc + 63) / 64, 128, 0, stream>>>(lX, lNorm, lWb, lBias, nc, lY);
    } else {
        k_infer_f32<<<(nc + 127) / 128, 128, 0, stream>>>(lX, lNorm, lW, nc, lY);
    }
    k_apply_prediction<<<(nc + 127) / 128, 128, 0, stream>>>(B, C[cur], nc, lY, P.friction_override,
                                                             (float)P.friction, lScope, bSlotOf, bLam, bLamL);
    AM_LAUNCHED(2);
    return AM_OK;
}

int Ctx::learnedPackInference() {
    k_pack_bf16<<<(NH * NH + 255) / 256, 256, 0, stream>>>(lW, lWb, lBias);
    AM_LAUNCHED(1);
    return syncErr();
}

// standardisation of the recorded features (mean, 1/std)
int Ctx::learnedNormalise() {
    int n = lDn;
    std::vector<float> X((size_t)n * NIN);
    cudaMemcpyAsync(X.data(), lDX, sizeof(float) * X.size(), cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    std::vector<float> nm(2 * NIN);
    for (int k = 0; k < NIN; k++) {
        double s = 0, s2 = 0;
        for (int i = 0; i < n; i++) { double v = X[(size_t)i * NIN + k]; s += v; s2 += v * v; }
        double m = n ? s / n : 0, var = n ? s2 / n - m * m : 1;
        nm[k] = (float)m;
        nm[NIN + k] = (float)(var > 1e-12 ? 1.0 / std::sqrt(var) : 1.0);
    }
    cudaMemcpyAsync(lNorm, nm.data(), sizeof(float) * 2 * NIN, cudaMemcpyHostToDevice, stream);
    return syncErr();
}

// mini-batch Adam on the recorded set; returns the mean loss of the last epoch
int Ctx::learnedTrain(int epochs, int batch, float lr, float* lastLoss, int normalise) {
    lReady = false;   // set again once the trained weights are packed
    int r = learnedInit();
    if (r) return r;
    int n = lDn;
    if (n < batch) { err = "not enough recorded samples"; return AM_E_STATE; }
    if (normalise && (r = learnedNormalise())) return r;
    if (batch > lTrainCap) {
        if (alloc(&lZ1, (size_t)NH * batch) || alloc(&lZ2, (size_t)NH * batch) || alloc(&lYh, (size_t)NOUT * batch) ||
            alloc(&lXN, (size_t)NIN * batch) || alloc(&lA1, (size_t)NH * batch) || alloc(&lA2, (size_t)NH * batch) ||
            alloc(&lD1, (size_t)NH * batch) || alloc(&lD2, (size_t)NH * batch) || alloc(&lDYb, (size_t)NOUT * batch))
            return AM_E_CUDA;
        lTrainCap = batch;
    }
    if (n > lIdxCap) {
        if (alloc(&lIdx, n)) return AM_E_CUDA;
        lIdxCap = n;
    }
    std::vector<int> perm(n);
    unsigned st = 777u;
    float el = 0.f;
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) {   // Fisher-Yates with a fixed LCG
            st = st * 1664525u + 1013904223u;
            int j = (int)(st % (unsigned)(i + 1));
            std::swap(perm[i], perm[j]);
        }
        cudaMemcpyAsync(lIdx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
        cudaMemsetAsync(lLoss, 0, sizeof(float), stream);
        int nb = n / batch;
        for (int b = 0; b < nb; b++) {
            const int* idx = lIdx + (size_t)b * batch;
            cudaMemsetAsync(lG, 0, sizeof(float) * NPAR, stream);
            k_fwd<<<(batch + 127) / 128, 128, 0, stream>>>(lDX, lNorm, lW, idx, batch, lZ1, lZ2, lYh);
            k_bwd_delta<<<(batch + 127) / 128, 128, 0, stream>>>(lDX, lDY, lNorm, lW, idx, batch, lZ1, lZ2, lYh, lXN,
                                                                 lA1, lA2, lD1, lD2, lDYb, lLoss);
            k_bwd_grad<<<dim3((NPAR + 127) / 128, (batch + GCH - 1) / GCH), 128, 0, stream>>>(lXN, lA1, lA2, lD1, lD2,
                                                                                             lDYb, batch, lG);
            lAdamT++;
            float c1 = 1.f / (1.f - std::pow(0.9f, (float)lAdamT)), c2 = 1.f / (1.f - std::pow(0.999f, (float)lAdamT));
            k_adam<<<(NPAR + 255) / 256, 256, 0, stream>>>(lW, lG, lM, lV, NPAR, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
            AM_LAUNCHED(4);
        }
        float ls = 0;
        cudaMemcpyAsync(&ls, lLoss, sizeof(float), cudaMemcpyDeviceToHost, stream);
        if ((r = syncErr())) return r;
        el = ls / (float)nb;
    }
    if (lastLoss) *lastLoss = el;
    if ((r = learnedPackInference())) return r;
    lReady = true;
    return AM_OK;
}

// loss and gradients of the current weights on host samples (test hook)
int Ctx::learnedGrad(const float* X, const float* Y, int n, float* grad, float* loss) {
    int r = learnedInit();
    if (r) return r;
    float *dX = nullptr, *dY = nullptr, *z1 = nullptr, *z2 = nullptr, *yh = nullptr, *xn = nullptr, *a1 = nullptr,
          *a2 = nullptr, *d1 = nullptr, *d2 = nullptr, *dyb = nullptr;
    if (tmpAlloc(&dX, (size_t)NIN * n) || tmpAlloc(&dY, (size_t)NOUT * n) || tmpAlloc(&z1, (size_t)NH * n) ||
        tmpAlloc(&z2, (size_t)NH * n) || tmpAlloc(&yh, (size_t)NOUT * n) || tmpAlloc(&xn, (size_t)NIN * n) ||
        tmpAlloc(&a1, (size_t)NH * n) || tmpAlloc(&a2, (size_t)NH * n) || tmpAlloc(&d1, (size_t)NH * n) ||
        tmpAlloc(&d2, (size_t)NH * n) || tmpAlloc(&dyb, (size_t)NOUT * n))
        return tmpFree(AM_E_CUDA);
    cudaMemcpyAsync(dX, X, sizeof(float) * NIN * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(dY, Y, sizeof(float) * NOUT * n, cudaMemcpyHostToDevice, stream);
    cudaMemsetAsync(lG, 0, sizeof(float) * NPAR, stream);
    cudaMemsetAsync(lLoss, 0, sizeof(float), stream);
    k_fwd<<<(n + 127) / 128, 128, 0, stream>>>(dX, lNorm, lW, nullptr, n, z1, z2, yh);
    k_bwd_delta<<<(n + 127) / 128, 128, 0, stream>>>(dX, dY, lNorm, lW, nullptr, n, z1, z2, yh, xn, a1, a2, d1, d2, dyb,
                                                     lLoss);
    k_bwd_grad<<<dim3((NPAR + 127) / 128, (n + GCH - 1) / GCH), 128, 0, stream>>>(xn, a1, a2, d1, d2, dyb, n, lG);
    AM_LAUNCHED(3);
    cudaMemcpyAsync(grad, lG, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(loss, lLoss, sizeof(float), cudaMemcpyDeviceToHost, stream);
    return tmpFree(syncErr());
}

int Ctx::learnedInfer(const float* X, int n, float* out, int tensorCores) {
    int r = learnedInit();
    if (r) return r;
    if ((r = learnedPackInference())) return r;
    float *dX = nullptr, *dO = nullptr;
    if (tmpAlloc(&dX, (size_t)NIN * n) || tmpAlloc(&dO, (size_t)NOUT * n)) return tmpFree(AM_E_CUDA);
    cudaMemcpyAsync(dX, X, sizeof(float) * NIN * n, cudaMemcpyHostToDevice, stream);
    if (tensorCores) k_infer_bf16<<<(n + 63) / 64, 128, 0, stream>>>(dX, lNorm, lWb, lBias, n, dO);
    else k_infer_f32<<<(n + 127) / 128, 128, 0, stream>>>(dX, lNorm, lW, n, dO);
    AM_LAUNCHED(1);
    cudaMemcpyAsync(out, dO, sizeof(float) * NOUT * n, cudaMemcpyDeviceToHost, stream);
    return tmpFree(syncErr());
}

int Ctx::learnedWeights(float* w, const float* in, float* norm, const float* normIn) {
    int r = learnedInit();
    if (r) return r;
    if (in) cudaMemcpyAsync(lW, in, sizeof(float) * NPAR, cudaMemcpyHostToDevice, stream);
    if (normIn) cudaMemcpyAsync(lNorm, normIn, sizeof(float) * 2 * NIN, cudaMemcpyHostToDevice, stream);
    if (w) cudaMemcpyAsync(w, lW, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, stream);
    if (norm) cudaMemcpyAsync(norm, lNorm, sizeof(float) * 2 * NIN, cudaMemcpyDeviceToHost, stream);
    if ((r = syncErr())) return r;
    if (!in) return AM_OK;
    lReady = false;
    if ((r = learnedPackInference())) return r;
    lReady = true;
    return AM_OK;
}

int Ctx::learnedCollect(int enable, int capacity) {
    int r = learnedInit();
    if (r) return r;
    lCollect = enable;
    if (enable && capacity > lDcap) {
        if (alloc(&lDX, (size_t)NIN * capacity) || alloc(&lDY, (size_t)NOUT * capacity)) return AM_E_CUDA;
        lDcap = capacity;
        lDn = 0;
    }
    return AM_OK;
}

// temporaries of the host-array hooks, freed before they return
template <class T>
int Ctx::tmpAlloc(T** p, size_t n) {
    if (cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
        err = "cudaMalloc failed";
        return AM_E_CUDA;
    }
    tmps.push_back((void*)*p);
    return AM_OK;
}

int Ctx::tmpFree(int r) {
    cudaStreamSynchronize(stream);
    for (void* q : tmps) cudaFree(q);
    tmps.clear();
    return r;
}

// ---------------------------------------------------------------------------
// Inference without allocation.  The rows pass through one fixed device
// scratch per device (AM_NOALLOC_MAX_ROWS rows of 24 input and 3 output
// floats, 7.1 MB) instead of the per-call temporaries of learnedInfer.  The
// scratch address is looked up once per device, on the first call made with
// that device current.  No part of the scratch needs to start at zero: every
// row a call reads was written by the same call's host-to-device copy.  Two
// calls that overlap in time on one device (any thread, stream or context)
// share the scratch and race.
static const int NOALLOC_ROWS = AM_NOALLOC_MAX_ROWS;
static const int NOALLOC_MAX_DEVICES = 64;
static __device__ __align__(256) float g_noalloc_scratch[(size_t)NOALLOC_ROWS * (NIN + NOUT)];
static float* g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// the scratch of device `dev`, which must be the current device (the symbol
// lookup resolves against the current device)
static float* noalloc_scratch(int dev) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return nullptr;
        g_noalloc_ptr[dev] = (float*)p;
    }
    return g_noalloc_ptr[dev];
}

// Same results as learnedInfer.  Status only (the context's error text is not
// touched, so a rejected call allocates nothing either).
int Ctx::learnedInferNoAlloc(const float* X, int n, float* out, int tensorCores) {
    if (n > NOALLOC_ROWS) return AM_E_CAPACITY;
    if (!lReady) return AM_E_STATE;   // weights are set up (and packed) by am_learned_use / _weights / _train
    // the scratch and the kernels belong to the context's device, which must
    // be the current one
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != device) return AM_E_STATE;
    float* base = noalloc_scratch(device);
    if (!base) return AM_E_CUDA;
    float* dX = base;
    float* dO = base + (size_t)NOALLOC_ROWS * NIN;
    if (cudaMemcpyAsync(dX, X, sizeof(float) * NIN * (size_t)n, cudaMemcpyHostToDevice, stream) != cudaSuccess)
        return AM_E_CUDA;
    if (tensorCores) k_infer_bf16<<<(n + 63) / 64, 128, 0, stream>>>(dX, lNorm, lWb, lBias, n, dO);
    else k_infer_f32<<<(n + 127) / 128, 128, 0, stream>>>(dX, lNorm, lW, n, dO);
    AM_LAUNCHED(1);
    if (cudaGetLastError() != cudaSuccess) return AM_E_CUDA;
    if (cudaMemcpyAsync(out, dO, sizeof(float) * NOUT * (size_t)n, cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return AM_E_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return AM_E_CUDA;
    return AM_OK;
}

int learned_num_params() { return NPAR; }

}  // namespace am
