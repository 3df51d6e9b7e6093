// batch.cu -- many independent scenes solved by one persistent launch.
//
// The scenes' bodies are concatenated (scene s owns body slots
// [sceneBodyOff[s], sceneBodyOff[s+1])); the collision pipeline runs on the
// whole batch with the broad phase restricted to pairs inside one scene, so
// every scene's contacts and body-pair groups are contiguous runs.  The solve
// then runs one CTA per scene:
//   * the scene's body delta-v lives in shared memory (FP32) for the whole
//     solve, so no delta-v traffic reaches HBM;
//   * the scene's body-pair groups are coloured inside the CTA (independent
//     set rounds over scene-local body indices);
//   * every contact is packed into a 64-float record (J, jinv J.w for both
//     bodies, b, D, 1/(D + c), mu, local body ids) read with 128-bit loads;
//   * each sweep walks the colours with __syncthreads between them; every
//     `check` sweeps the CTA evaluates the natural-map residual of its scene
//     and stops when it is below the target (or at the iteration cap);
//   * multipliers go back to the FP64 contact arrays and delta-v to the FP64
//     body arrays for integration.
// This is the FP32 path of the batched workload (the single-scene drop-in
// stays FP64); threads per CTA are chosen by the autotuner in Ctx.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

static const int REC = 64;      // floats per packed contact record
static const int MAXCB = 64;    // colours per scene

// Packed record (floats): row r = 0..2 occupies [20r, 20r + 20):
//   [20r .. 20r+11] J (a.v, a.w, b.v, b.w), [20r+12 .. 20r+14] jinv_a a.w,
//   [20r+15 .. 20r+17] jinv_b b.w, [20r+18] b, [20r+19] 1/(D + c);
// [60 .. 62] D of the three rows, [63] mu.  Scene-local body ids live in a
// separate int2 array, the multipliers in a separate float array (the only
// per-sweep writes).

__global__ void k_scene_ranges(const DPairs P, int npairs, const int* sceneOf, int nScenes, int* pairOff) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > npairs) return;
    int sp = p < npairs ? sceneOf[P.a[p]] : nScenes;
    int sq = p > 0 ? sceneOf[P.a[p - 1]] : -1;
    for (int s = sq + 1; s <= sp; s++) pairOff[s] = p;
}

__global__ void k_batch_pack(DBodies B, DContacts C, int nc, const int* sceneOf, const int* sceneBodyOff,
                             double comp, int fo, double fv, float* rec, int2* lid, float* lamf) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int cap = C.cap;
    float r[REC];
    for (int q = 0; q < 3; q++) {
        for (int k = 0; k < 12; k++) r[20 * q + k] = (float)C.J[(12 * q + k) * cap + c];
        for (int k = 0; k < 3; k++) {
            r[20 * q + 12 + k] = (float)C.Ia[(3 * q + k) * cap + c];
            r[20 * q + 15 + k] = (float)C.Ib[(3 * q + k) * cap + c];
        }
        double D = C.bD[(3 + q) * cap + c];
        r[20 * q + 18] = (float)C.bD[q * cap + c];
        r[20 * q + 19] = (float)(1.0 / (D + comp));
        r[60 + q] = (float)D;
        lamf[3 * c + q] = (float)C.lam[q * cap + c];
    }
    double mu;
    if (fo) mu = fv;
    else {
        double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
        if (f1 < 0.2 || f2 < 0.2) mu = fmin(f1, f2);
        else if (f1 > 1. || f2 > 1.) mu = fmax(f1, f2);
        else mu = (f1 + f2) / 2.;
    }
    r[63] = (float)mu;
    float4* dst = reinterpret_cast<float4*>(rec + (size_t)REC * c);
    for (int k = 0; k < REC / 4; k++) dst[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
    int s1 = C.sb1[c], s2 = C.sb2[c];
    int base = sceneBodyOff[sceneOf[s1]];
    lid[c] = make_int2(s1 - base, s2 - base);
}

// Colour the groups (body pairs) of one scene, one CTA per scene:
// Jones-Plassmann rounds with first-fit colours.  Each round, an uncoloured
// group whose priority is the largest among the uncoloured groups at both of
// its (non-pinned) bodies takes the smallest colour not yet used at either
// body.  Selected groups of one round share no body, so the per-body colour
// masks need no atomics between them.  Priorities put groups with more
// contacts first (they then sit in the low colours), ties broken by a hash
// and made unique by the group index.
__global__ void k_batch_colour(DBodies B, DContacts C, DPairs P, const int* pairOff, const int* sceneBodyOff,
                               int* colourOf, int* gOrder, int* colOff, int maxBodies, DCount* dc) {
    extern __shared__ unsigned long long smemq[];
    unsigned long long* bodyMax = smemq;               // [maxBodies] largest uncoloured priority
    unsigned long long* used = smemq + maxBodies;      // [maxBodies] colours taken at the body
    __shared__ int s_left, s_full, s_cnt[MAXCB + 1];
    int s = blockIdx.x;
    int g0 = pairOff[s], g1 = pairOff[s + 1];
    int b0 = sceneBodyOff[s], nb = sceneBodyOff[s + 1] - b0;
    int t = threadIdx.x, T = blockDim.x;
    if (nb > maxBodies) { if (t == 0) dc->error = AM_E_CAPACITY; return; }
    for (int g = g0 + t; g < g1; g += T) colourOf[g] = P.count[g] > 0 ? -1 : -2;
    for (int k = t; k <= MAXCB; k += T) s_cnt[k] = 0;
    for (int b = t; b < nb; b += T) used[b] = 0ull;
    if (t == 0) s_full = 0;
    __syncthreads();
    auto prio = [&](int g) -> unsigned long long {
        unsigned h = (unsigned)g * 2654435761u;
        h ^= h >> 16;
        unsigned long long cnt = (unsigned long long)min(P.count[g], 255);
        return (cnt << 56) | ((unsigned long long)(h & 0xFFFFFFu) << 32) | (unsigned)(g - g0);
    };
    const int maxRounds = 1 << 16;
    for (int round = 0; round < maxRounds; round++) {
        for (int b = t; b < nb; b += T) bodyMax[b] = 0ull;
        if (t == 0) s_left = 0;
        __syncthreads();
        for (int g = g0 + t; g < g1; g += T) {
            if (colourOf[g] != -1) continue;
            int c = P.off[g];
            int s1 = C.sb1[c], s2 = C.sb2[c];
            unsigned long long pr = prio(g);
            if (!(B.flags[s1] & F_PINNED)) atomicMax(&bodyMax[s1 - b0], pr);
            if (!(B.flags[s2] & F_PINNED)) atomicMax(&bodyMax[s2 - b0], pr);
        }
        __syncthreads();
        for (int g = g0 + t; g < g1; g += T) {
            if (colourOf[g] != -1) continue;
            int c = P.off[g];
            int s1 = C.sb1[c], s2 = C.sb2[c];
            bool p1 = B.flags[s1] & F_PINNED, p2 = B.flags[s2] & F_PINNED;
            unsigned long long pr = prio(g);
            bool ok = (p1 || bodyMax[s1 - b0] == pr) && (p2 || bodyMax[s2 - b0] == pr);
            if (!ok) { atomicAdd(&s_left, 1); continue; }
            unsigned long long m = (p1 ? 0ull : used[s1 - b0]) | (p2 ? 0ull : used[s2 - b0]);
            if (m == ~0ull) { colourOf[g] = -2; s_full = 1; continue; }   // more than MAXCB colours needed
            int col = __ffsll((long long)~m) - 1;
            if (!p1) used[s1 - b0] |= 1ull << col;
            if (!p2) used[s2 - b0] |= 1ull << col;
            colourOf[g] = col;
            atomicAdd(&s_cnt[col], 1);
        }
        __syncthreads();
        int left = s_left;
        __syncthreads();
        if (left == 0) break;
    }
    __syncthreads();
    if (t == 0) {
        if (s_left || s_full) dc->error = AM_E_CAPACITY;
        int ncol = 0;
        for (int k = 0; k < MAXCB; k++) if (s_cnt[k]) ncol = k + 1;
        int run = g0;
        for (int k = 0; k < ncol; k++) { int n = s_cnt[k]; s_cnt[k] = run; colOff[s * (MAXCB + 1) + k] = run; run += n; }
        for (int k = ncol; k <= MAXCB; k++) colOff[s * (MAXCB + 1) + k] = run;
    }
    __syncthreads();
    for (int g = g0 + t; g < g1; g += T) {
        int c = colourOf[g];
        if (c >= 0) gOrder[atomicAdd(&s_cnt[c], 1)] = g;
    }
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void prefetch_l1(const float* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// J . dv of one row over the group's two bodies (record layout: a.v a.w b.v b.w
// in j0..j2), as two independent half sums
__device__ __forceinline__ float group_jdv(const float* a, const float* b, float4 j0, float4 j1, float4 j2) {
    float sa = j0.x * a[0] + j0.y * a[1] + j0.z * a[2] + j0.w * a[3] + j1.x * a[4] + j1.y * a[5];
    float sb = j1.z * b[0] + j1.w * b[1] + j2.x * b[2] + j2.y * b[3] + j2.z * b[4] + j2.w * b[5];
    return sa + sb;
}

// delta-v += (minv J.v, jinv J.w) * d for both bodies (i0, i1 hold jinv J.w)
__device__ __forceinline__ void group_update(float* a, float* b, float la, float lb, float d, float4 j0, float4 j1,
                                             float4 j2, float4 i0, float4 i1) {
    a[0] += la * j0.x; a[1] += la * j0.y; a[2] += la * j0.z;
    a[3] += d * i0.x; a[4] += d * i0.y; a[5] += d * i0.z;
    b[0] += lb * j1.z; b[1] += lb * j1.w; b[2] += lb * j2.x;
    b[3] += d * i0.w; b[4] += d * i1.x; b[5] += d * i1.y;
}

// one CTA per scene; dynamic smem: dv[6 * maxBodies] + minv[maxBodies]
__global__ void k_batch_sweep(DBodies B, DContacts C, DPairs P, const int* pairOff, const int* sceneBodyOff,
                              const int* gOrder, const int* colOff, const float* rec, const int2* lid, float* lamf,
                              int iters, float omega, float comp, float tolRel, int check, float slide,
                              int* sceneSweeps, float* sceneRes, DCount* dc, const float* lamAlt, int* sceneFall) {
    extern __shared__ float sm[];
    int s = blockIdx.x;
    int b0 = sceneBodyOff[s], nb = sceneBodyOff[s + 1] - b0;
    float* dv = sm;                 // [6 nb]
    float* mv = sm + 6 * nb;        // [nb]
    __shared__ float s_res, s_lam;
    __shared__ int s_stop;
    int t = threadIdx.x, T = blockDim.x;
    // pinned bodies get 0 here, the same test the colouring uses to let groups
    // of one colour share them
    for (int b = t; b < nb; b += T) mv[b] = (B.flags[b0 + b] & F_PINNED) ? 0.f : (float)B.minv[b0 + b];
    const int* co = colOff + s * (MAXCB + 1);
    int ncol = 0;
    while (ncol < MAXCB && co[ncol + 1] > co[ncol]) ncol++;
    int total = 0;
    float res = 0.f;
    // attempt 0 starts from lamf; with lamAlt given, a scene that misses the
    // residual target starts again from lamAlt (the learned start's fallback)
    const int attempts = (lamAlt && check > 0 && tolRel > 0.f) ? 2 : 1;
    for (int attempt = 0; attempt < attempts; attempt++) {
        if (attempt == 1) {
            if (res <= tolRel) break;   // uniform: res comes from shared memory
            for (int g = pairOff[s] + t; g < pairOff[s + 1]; g += T)
                for (int c = P.off[g]; c < P.off[g] + P.count[g]; c++)
                    for (int q = 0; q < 3; q++) lamf[3 * c + q] = lamAlt[3 * c + q];
            if (t == 0 && sceneFall) sceneFall[s] = 1;
        } else if (t == 0 && sceneFall) {
            sceneFall[s] = 0;
        }
        for (int b = t; b < nb; b += T)
            for (int k = 0; k < 6; k++) dv[6 * b + k] = 0.f;
        __syncthreads();
        // confidentWarmStart.  Every contact of a group acts on the same two
        // bodies, so their delta-v stays in registers for the whole group.
        for (int col = 0; col < ncol; col++) {
            for (int k = co[col] + t; k < co[col + 1]; k += T) {
                int g = gOrder[k];
                int c0 = P.off[g], c1 = c0 + P.count[g];
                int2 id = lid[c0];
                float a[6], b[6];
                for (int q = 0; q < 6; q++) { a[q] = dv[6 * id.x + q]; b[q] = dv[6 * id.y + q]; }
                float ma = mv[id.x], mb = mv[id.y];
                for (int c = c0; c < c1; c++) {
                    const float* R = rec + (size_t)REC * c;
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        float l = lamf[3 * c + q];
                        float4 j0 = ld4(R + 20 * q), j1 = ld4(R + 20 * q + 4), j2 = ld4(R + 20 * q + 8);
                        float4 i0 = ld4(R + 20 * q + 12), i1 = ld4(R + 20 * q + 16);
                        group_update(a, b, ma * l, mb * l, l, j0, j1, j2, i0, i1);
                    }
                }
                // pinned bodies (minv = 0) never change and may be shared within a colour
                if (ma != 0.f) for (int q = 0; q < 6; q++) dv[6 * id.x + q] = a[q];
                if (mb != 0.f) for (int q = 0; q < 6; q++) dv[6 * id.y + q] = b[q];
            }
            __syncthreads();
        }
        int done = 0;
        for (int it = 0; it < iters; it++) {
            bool last = (it == iters - 1);
            for (int col = 0; col < ncol; col++) {
                for (int k = co[col] + t; k < co[col + 1]; k += T) {
                    int g = gOrder[k];
                    int c0 = P.off[g], c1 = c0 + P.count[g];
                    int2 id = lid[c0];
                    float a[6], b[6];
                    for (int q = 0; q < 6; q++) { a[q] = dv[6 * id.x + q]; b[q] = dv[6 * id.y + q]; }
                    float ma = mv[id.x], mb = mv[id.y];
                    for (int c = c0; c < c1; c++) {
                        const float* R = rec + (size_t)REC * c;
                        float4 tail = ld4(R + 60);
                        float lam[3] = {lamf[3 * c], lamf[3 * c + 1], lamf[3 * c + 2]};
                        float l0 = lam[0];
#pragma unroll
                        for (int q = 0; q < 3; q++) {
                            float4 j0 = ld4(R + 20 * q), j1 = ld4(R + 20 * q + 4), j2 = ld4(R + 20 * q + 8);
                            float4 i0 = ld4(R + 20 * q + 12), i1 = ld4(R + 20 * q + 16);
                            float jd = group_jdv(a, b, j0, j1, j2);
                            float D = q == 0 ? tail.x : (q == 1 ? tail.y : tail.z);
                            float l = lam[q];
                            float nl = (D * l - omega * (i1.z + jd)) * i1.w;
                            if (q == 0) nl = fmaxf(nl, 0.f);
                            else { float lim = tail.w * l0; nl = fminf(fmaxf(nl, -lim), lim); }
                            float d = nl - l;
                            if (q == 0) l0 = nl;
                            lam[q] = nl;
                            group_update(a, b, ma * d, mb * d, d, j0, j1, j2, i0, i1);
                        }
                        lamf[3 * c] = lam[0]; lamf[3 * c + 1] = lam[1]; lamf[3 * c + 2] = lam[2];
                    }
                    if (ma != 0.f) for (int q = 0; q < 6; q++) dv[6 * id.x + q] = a[q];
                    if (mb != 0.f) for (int q = 0; q < 6; q++) dv[6 * id.y + q] = b[q];
                }
                // while the colour drains, pull this thread's first group of the
                // next colour (or of colour 0 for the next sweep) into L1
                {
                    int nc2 = col + 1 < ncol ? col + 1 : 0;
                    int k2 = co[nc2] + t;
                    if (k2 < co[nc2 + 1]) {
                        int g2 = gOrder[k2];
                        const float* R2 = rec + (size_t)REC * P.off[g2];
                        int lines = 2 * P.count[g2];
                        for (int q = 0; q < lines; q++) prefetch_l1(R2 + 32 * q);
                        prefetch_l1(lamf + 3 * P.off[g2]);
                    }
                }
                __syncthreads();
            }
            done = it + 1;
            if (check > 0 && (done % check == 0 || done == iters)) {
                // natural-map residual of the scene at the current state
                if (t == 0) { s_res = 0.f; s_lam = 0.f; }
                __syncthreads();
                float rmax = 0.f, lmax = 0.f;
                for (int g = pairOff[s] + t; g < pairOff[s + 1]; g += T)
                    for (int c = P.off[g]; c < P.off[g] + P.count[g]; c++) {
                        int2 id = lid[c];
                        const float* R = rec + (size_t)REC * c;
                        const float* da = dv + 6 * id.x;
                        const float* db = dv + 6 * id.y;
                        float4 tail = ld4(R + 60);
                        float l0 = lamf[3 * c];
                        for (int q = 0; q < 3; q++) {
                            float4 j0 = ld4(R + 20 * q), j1 = ld4(R + 20 * q + 4), j2 = ld4(R + 20 * q + 8);
                            float4 i1 = ld4(R + 20 * q + 16);
                            float jd = j0.x * da[0] + j0.y * da[1] + j0.z * da[2] + j0.w * da[3] + j1.x * da[4] +
                                       j1.y * da[5] + j1.z * db[0] + j1.w * db[1] + j2.x * db[2] + j2.y * db[3] +
                                       j2.z * db[4] + j2.w * db[5];
                            float l = lamf[3 * c + q];
                            float w = i1.z + jd + comp * l;
                            float z = l - w * i1.w;
                            if (q == 0) z = fmaxf(z, 0.f);
                            else { float lim = tail.w * l0; z = fminf(fmaxf(z, -lim), lim); }
                            rmax = fmaxf(rmax, fabsf(l - z));
                            lmax = fmaxf(lmax, fabsf(l));
                        }
                    }
                atomicMax(reinterpret_cast<int*>(&s_res), __float_as_int(rmax));
                atomicMax(reinterpret_cast<int*>(&s_lam), __float_as_int(lmax));
                __syncthreads();
                res = s_res / fmaxf(1.f, s_lam);
                if (t == 0) s_stop = (res <= tolRel) ? 1 : 0;
                __syncthreads();
                if (s_stop) break;
            }
        }
        total += done;
    }
    // contact state after the final sweep (Contact.updateContactState)
    for (int g = pairOff[s] + t; g < pairOff[s + 1]; g += T)
        for (int c = P.off[g]; c < P.off[g] + P.count[g]; c++) {
            int2 id = lid[c];
            const float* R = rec + (size_t)REC * c;
            const float* da = dv + 6 * id.x;
            const float* db = dv + 6 * id.y;
            float w[2];
            for (int q = 1; q < 3; q++) {
                float4 j0 = ld4(R + 20 * q), j1 = ld4(R + 20 * q + 4), j2 = ld4(R + 20 * q + 8);
                float4 i1 = ld4(R + 20 * q + 16);
                w[q - 1] = i1.z + j0.x * da[0] + j0.y * da[1] + j0.z * da[2] + j0.w * da[3] + j1.x * da[4] +
                           j1.y * da[5] + j1.z * db[0] + j1.w * db[1] + j2.x * db[2] + j2.y * db[3] +
                           j2.z * db[4] + j2.w * db[5];
            }
            int cap = C.cap;
            float l0 = lamf[3 * c];
            int st;
            if (fabsf(l0) <= 1e-14f) st = AM_STATE_BROKEN;
            else if (fabsf(w[0]) > slide || fabsf(w[1]) > slide) st = AM_STATE_ONEDGE;
            else st = AM_STATE_CLEAR;
            C.state[c] = st;
            for (int q = 0; q < 3; q++) C.lam[q * cap + c] = (double)lamf[3 * c + q];
        }
    for (int b = t; b < nb; b += T)
        for (int k = 0; k < 6; k++) B.dv[6 * (b0 + b) + k] = (double)dv[6 * b + k];
    if (t == 0) { sceneSweeps[s] = total; sceneRes[s] = res; }
}

const void* batch_sweep_kernel() { return (const void*)k_batch_sweep; }

int Ctx::batchSolve(double dt) {
    int r;
    int nc = nContacts, np = nPairs, S = nScenes;
    if (nc <= 0) return AM_OK;
    double comp = P.enable_compliance ? P.compliance : 0.;
    launch_solve_prep(B, C[cur], nc, dt, P.feedback_stiffness, false, P.restitution_override, P.restitution,
                      P.warm_start ? 1 : 0, stream);
    if (nc > bRecCap) {
        int cap = std::max(nc + nc / 2, 4096);
        if (alloc(&bRec, (size_t)REC * cap) || alloc(&bLid, cap) || alloc(&bLam, 3 * (size_t)cap) ||
            alloc(&bLamL, 3 * (size_t)cap))
            return AM_E_CUDA;
        bRecCap = cap;
    }
    if (np > bPairCap) {
        int cap = std::max(np + np / 2, 4096);
        if (alloc(&bColour, cap) || alloc(&bOrder, cap)) return AM_E_CUDA;
        bPairCap = cap;
    }
    k_scene_ranges<<<(np + 1 + 255) / 256, 256, 0, stream>>>(PR, np, sceneOfDev, S, bPairOff);
    k_batch_pack<<<(nc + 127) / 128, 128, 0, stream>>>(B, C[cur], nc, sceneOfDev, sceneBodyOffDev, comp,
                                                     P.friction_override, P.friction, bRec, bLid, bLam);
    size_t csm = 2 * sizeof(unsigned long long) * (size_t)maxSceneBodies;
    k_batch_colour<<<S, 256, csm, stream>>>(B, C[cur], PR, bPairOff, sceneBodyOffDev, bColour, bOrder, bColOff,
                                            maxSceneBodies, dc);
    size_t ssm = sizeof(float) * 7 * (size_t)maxSceneBodies;
    int threads = batchThreads > 0 ? batchThreads : 128;
    if (evA) cudaEventRecord(evA, stream);
    if (lUse || lCollect) {
        if ((r = learnedFeatures(dt))) return r;
    }
    float* lamStart = bLam;
    const float* lamAlt = nullptr;
    if (lUse) {
        // learned start in bLamL; the plain previous-frame start stays in bLam
        // as the in-kernel fallback
        if ((r = learnedPredict(lUse == 1))) return r;
        lamStart = bLamL;
        lamAlt = bLam;
    }
    k_batch_sweep<<<S, threads, ssm, stream>>>(B, C[cur], PR, bPairOff, sceneBodyOffDev, bOrder, bColOff, bRec,
                                               bLid, lamStart, P.iterations, (float)P.omega, (float)comp,
                                               (float)batchTol, batchCheck, (float)P.sliding_threshold,
                                               bSweeps, bRes, dc, lamAlt, bFall);
    AM_LAUNCHED(4);
    if (evB) { cudaEventRecord(evB, stream); pgsPending = true; }
    if (lCollect && (r = learnedRecord())) return r;
    return AM_OK;
}

// contacts of each scene times its sweeps (contacts of a scene are contiguous)
__global__ void k_scene_cs(DPairs P, int npairs, int nc, const int* pairOff, const int* sweeps, int nScenes,
                           long long* out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nScenes) return;
    int a = pairOff[s] < npairs ? P.off[pairOff[s]] : nc;
    int b = pairOff[s + 1] < npairs ? P.off[pairOff[s + 1]] : nc;
    out[s] = (long long)(b - a) * sweeps[s];
}

// colours per scene of the last colouring (colours are contiguous from 0)
int Ctx::batchColours(int* out) {
    std::vector<int> co((size_t)nScenes * (MAXCB + 1));
    cudaMemcpyAsync(co.data(), bColOff, sizeof(int) * co.size(), cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    for (int s = 0; s < nScenes; s++) {
        const int* c = co.data() + (size_t)s * (MAXCB + 1);
        int n = 0;
        while (n < MAXCB && c[n + 1] > c[n]) n++;
        out[s] = n;
    }
    return AM_OK;
}

int Ctx::batchStats() {
    std::vector<int> sw(nScenes), fl(nScenes);
    std::vector<float> rs(nScenes);
    std::vector<long long> cs(nScenes);
    if (!bCS && alloc(&bCS, nScenes)) return AM_E_CUDA;
    k_scene_cs<<<(nScenes + 127) / 128, 128, 0, stream>>>(PR, nPairs, nContacts, bPairOff, bSweeps, nScenes, bCS);
    AM_LAUNCHED(1);
    cudaMemcpyAsync(cs.data(), bCS, sizeof(long long) * nScenes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(sw.data(), bSweeps, sizeof(int) * nScenes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(rs.data(), bRes, sizeof(float) * nScenes, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(fl.data(), bFall, sizeof(int) * nScenes, cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    long long tot = 0;
    int mx = 0;
    float rmax = 0.f;
    int conv = 0, fall = 0;
    for (int s = 0; s < nScenes; s++) {
        tot += sw[s];
        mx = std::max(mx, sw[s]);
        rmax = std::max(rmax, rs[s]);
        conv += rs[s] <= batchTol ? 1 : 0;
        fall += fl[s];
    }
    lFallbackScenes = lUse ? fall : 0;
    batchSweepsTotal = tot;
    batchContactSweepsLast = 0;
    for (long long v : cs) batchContactSweepsLast += v;
    stats.sweeps = mx;
    stats.residual_rel = rmax;
    batchConverged = conv;
    return AM_OK;
}

}  // namespace am

namespace am {

// Load a batch of independent scenes: bodies and tree nodes are concatenated
// with offsets; body slot i of scene s is sceneBodyOff[s] + i.
int Ctx::setBatch(const am_scene* sc, int n) {
    std::vector<int> type, pinned, root, c0, nch;
    std::vector<double> x, R, v, w, mass, inertia, fr, re, shape, nc, nr;
    std::vector<int> bodyOff(n + 1, 0), sceneOf;
    int nodeBase = 0;
    maxSceneBodies = 0;
    for (int s = 0; s < n; s++) {
        const am_scene& a = sc[s];
        bodyOff[s + 1] = bodyOff[s] + a.n_bodies;
        maxSceneBodies = std::max(maxSceneBodies, a.n_bodies);
        for (int i = 0; i < a.n_bodies; i++) {
            type.push_back(a.type[i]); pinned.push_back(a.pinned[i]);
            root.push_back(a.body_root[i] >= 0 ? a.body_root[i] + nodeBase : -1);
            for (int k = 0; k < 3; k++) { x.push_back(a.x[3 * i + k]); v.push_back(a.v[3 * i + k]); w.push_back(a.omega[3 * i + k]); }
            for (int k = 0; k < 9; k++) { R.push_back(a.R[9 * i + k]); inertia.push_back(a.inertia[9 * i + k]); }
            for (int k = 0; k < 4; k++) shape.push_back(a.shape[4 * i + k]);
            mass.push_back(a.mass[i]); fr.push_back(a.friction[i]); re.push_back(a.restitution[i]);
            sceneOf.push_back(s);
        }
        for (int k = 0; k < a.n_nodes; k++) {
            for (int q = 0; q < 3; q++) nc.push_back(a.node_c[3 * k + q]);
            nr.push_back(a.node_r[k]);
            c0.push_back(a.node_child0[k] >= 0 ? a.node_child0[k] + nodeBase : -1);
            nch.push_back(a.node_nchild[k]);
        }
        nodeBase += a.n_nodes;
    }
    am_scene all;
    all.n_bodies = bodyOff[n];
    all.type = type.data(); all.pinned = pinned.data(); all.x = x.data(); all.R = R.data(); all.v = v.data();
    all.omega = w.data(); all.mass = mass.data(); all.inertia = inertia.data(); all.friction = fr.data();
    all.restitution = re.data(); all.shape = shape.data(); all.n_nodes = nodeBase; all.body_root = root.data();
    all.node_c = nc.data(); all.node_r = nr.data(); all.node_child0 = c0.data(); all.node_nchild = nch.data();
    int r = setScene(all);
    if (r) return r;
    nScenes = n;
    int cap = host.cap;
    std::vector<int> sOf(cap, n), tEnd(all.n_bodies);
    for (int i = 0; i < all.n_bodies; i++) { sOf[i] = sceneOf[i]; tEnd[i] = bodyOff[sceneOf[i] + 1]; }
    bCS = nullptr;
    if (alloc(&sceneOfDev, cap) || alloc(&sceneBodyOffDev, n + 1) || alloc(&topEnd, all.n_bodies) ||
        alloc(&bPairOff, n + 1) || alloc(&bColOff, (size_t)n * (MAXCB + 1)) || alloc(&bSweeps, n) || alloc(&bRes, n) ||
        alloc(&bFall, n))
        return AM_E_CUDA;
    cudaMemsetAsync(bFall, 0, sizeof(int) * n, stream);
    cudaMemcpyAsync(sceneOfDev, sOf.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(sceneBodyOffDev, bodyOff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(topEnd, tEnd.data(), sizeof(int) * all.n_bodies, cudaMemcpyHostToDevice, stream);
    size_t ssm = sizeof(float) * 7 * (size_t)maxSceneBodies;
    if (ssm > 48 * 1024) cudaFuncSetAttribute(batch_sweep_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm);
    size_t csm = 2 * sizeof(unsigned long long) * (size_t)maxSceneBodies;
    if (csm > 48 * 1024)
        cudaFuncSetAttribute((const void*)k_batch_colour, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm);
    return syncErr();
}

// Picks the CTA size of the scene solve: every candidate runs a few sweeps
// from the same packed state (multipliers restored between candidates) and
// the fastest per sweep wins.
int Ctx::batchAutotune(double dt) {
    (void)dt;
    const int cand[4] = {64, 128, 256, 512};
    double comp = P.enable_compliance ? P.compliance : 0.;
    int nc = nContacts;
    float* save = nullptr;
    if (alloc(&save, 3 * (size_t)nc)) return AM_E_CUDA;
    cudaMemcpyAsync(save, bLam, sizeof(float) * 3 * nc, cudaMemcpyDeviceToDevice, stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    size_t ssm = sizeof(float) * 7 * (size_t)maxSceneBodies;
    float best = 1e30f;
    int bestT = 128;
    tuneMs.clear();
    for (int k = 0; k < 4; k++) {
        int T = cand[k];
        cudaMemcpyAsync(bLam, save, sizeof(float) * 3 * nc, cudaMemcpyDeviceToDevice, stream);
        cudaEventRecord(e0, stream);
        k_batch_sweep<<<nScenes, T, ssm, stream>>>(B, C[cur], PR, bPairOff, sceneBodyOffDev, bOrder, bColOff, bRec,
                                                   bLid, bLam, 8, (float)P.omega, (float)comp, 0.f, 0,
                                                   (float)P.sliding_threshold, bSweeps, bRes, dc, nullptr, nullptr);
        cudaEventRecord(e1, stream);
        AM_LAUNCHED(1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        tuneMs.push_back(ms);
        if (ms < best) { best = ms; bestT = T; }
    }
    cudaMemcpyAsync(bLam, save, sizeof(float) * 3 * nc, cudaMemcpyDeviceToDevice, stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    batchThreads = bestT;
    return syncErr();
}

// RigidBodySystem.advanceTime for every scene of the batch (merging off)
int Ctx::stepBatch(double dt) {
    int r;
    if ((r = beginStep(0))) return r;
    if ((r = collisionDetection())) return r;
    if ((r = warmStart())) return r;
    if ((r = wake())) return r;
    if (!evA) { cudaEventCreate(&evA); cudaEventCreate(&evB); }
    if (batchThreads == 0 && nContacts > 0) {
        // pack once to tune on real data, then solve with the chosen size
        int keep = batchThreads;
        batchThreads = 128;
        if ((r = batchSolve(dt))) return r;
        if ((r = syncErr())) return r;
        pgsPending = false;
        batchThreads = keep;
        // restore the warm-start multipliers the solve consumed and retune
        if ((r = batchAutotune(dt))) return r;
        cudaMemsetAsync(B.dv, 0, sizeof(double) * 6 * host.cap, stream);
    }
    if ((r = batchSolve(dt))) return r;
    if ((r = finishStep(dt))) return r;
    if ((r = readCounts())) return r;
    if (pgsPending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, evA, evB) == cudaSuccess) {
            perf.pgs_ms += ms;
            perf.pgs_launches += 1;
        }
        pgsPending = false;
    }
    if ((r = batchStats())) return r;
    perf.contact_sweeps += batchContactSweepsLast;
    perf.steps++;
    stats.n_contacts = nContacts;
    return AM_OK;
}

}  // namespace am
