// pgs_fast.cu -- coloured projected Gauss-Seidel, FP64, latency-optimised.
//
// GB300 issues one FP64 warp instruction per ~64 cycles per SM sub-partition
// (1.2 TFLOP/s FP64 vs 68 TFLOP/s FP32, measured), so a Gauss-Seidel sweep is
// bound by the length of its dependent FP64 instruction chain, not by HBM.
// This kernel shortens that chain:
//   * one 16-lane half-warp per body-pair group; lane k (k < 12) owns Jacobian
//     entry k of a row (a.v xyz, a.w xyz, b.v xyz, b.w xyz) and the matching
//     delta-v component, held in a register for the whole group (the group's
//     two bodies are touched by no other group of the same colour);
//   * J . dv is a 4-level shuffle tree, the delta-v update a single FMA per
//     lane with M^-1 J^T precomputed per contact;
//   * 1/(D + c) is precomputed per row, so the projected update needs no
//     division.
// Contacts of a group stay sequential in list order; colours are separated
// by the bounded grid barrier.  Results equal the reference's fixed point,
// not its per-sweep bits (AM_ORDER_COLOURED); this translation unit is
// compiled with FMA contraction on.
#include <cuda_runtime.h>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

// per-contact precompute: Mj[36] (M^-1 J^T entries, row-major by row then
// lane k) and invD[3]
__global__ void k_fast_prep(DBodies B, DContacts C, int nc, double comp, double* Mj, double* invD, int cap) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int ccap = C.cap;
    int s1 = C.sb1[c], s2 = C.sb2[c];
    double m1 = B.minv[s1], m2 = B.minv[s2];
    for (int r = 0; r < 3; r++) {
        for (int k = 0; k < 3; k++) {
            Mj[(12 * r + k) * cap + c] = m1 * C.J[(12 * r + k) * ccap + c];          // a.v
            Mj[(12 * r + 3 + k) * cap + c] = C.Ia[(3 * r + k) * ccap + c];           // jinv1 a.w
            Mj[(12 * r + 6 + k) * cap + c] = m2 * C.J[(12 * r + 6 + k) * ccap + c];  // b.v
            Mj[(12 * r + 9 + k) * cap + c] = C.Ib[(3 * r + k) * ccap + c];           // jinv2 b.w
        }
        invD[r * cap + c] = 1.0 / (C.bD[(3 + r) * ccap + c] + comp);
    }
}

__device__ __forceinline__ double hw_sum(double v, unsigned mask) {
    v += __shfl_xor_sync(mask, v, 8, 16);
    v += __shfl_xor_sync(mask, v, 4, 16);
    v += __shfl_xor_sync(mask, v, 2, 16);
    v += __shfl_xor_sync(mask, v, 1, 16);
    return v;
}

__device__ __forceinline__ bool grid_barrier_f(DCount* dc, int nblocks) {
    if (nblocks == 1) {   // one block: the block barrier orders global memory too
        __syncthreads();
        return *(volatile int*)&dc->error == 0;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile int* gen = &dc->bar_gen;
        int g0 = *gen;
        __threadfence();
        int arrived = atomicAdd(&dc->bar_count, 1);
        if (arrived == nblocks - 1) {
            dc->bar_count = 0;
            __threadfence();
            atomicAdd(&dc->bar_gen, 1);
        } else {
            long long spins = 0;
            while (*gen == g0) {
                if (++spins > (1ll << 24)) { atomicExch(&dc->error, AM_E_TIMEOUT); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&dc->error == 0;
}

__device__ __forceinline__ double mu_fast(const DBodies& B, const DContacts& C, int c, int fo, double fv) {
    if (fo) return fv;
    double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
    if (f1 < 0.2 || f2 < 0.2) return fmin(f1, f2);
    if (f1 > 1. || f2 > 1.) return fmax(f1, f2);
    return (f1 + f2) / 2.;
}

__global__ void __launch_bounds__(128) k_pgs_fast(DBodies B, DContacts C, DPairs P, const int* groupOrder,
                                                   const int* colourOff, int ncol, int iters, double omega,
                                                   double tol, int early, int fo, double fv, double slide,
                                                   const double* Mj, const double* invD, int mcap, DCount* dc,
                                                   double comp, double resTol, int check) {
    const int nblocks = gridDim.x;
    const int lane = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const unsigned mask = 0xFFFFu << (16 * half);
    const int hw = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    const int nhw = (nblocks * blockDim.x) >> 4;
    const int ccap = C.cap;
    const bool act = lane < 12;
    const int side = lane / 6;         // 0: body 1, 1: body 2
    const int comp6 = lane % 6;        // v xyz, w xyz

    // confidentWarmStart, colour by colour
    for (int col = 0; col < ncol; col++) {
        for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
            int g = groupOrder[k];
            int c0 = P.off[g], n = P.count[g];
            int body = act ? (side == 0 ? C.sb1[c0] : C.sb2[c0]) : 0;
            double* dvp = B.dv + 6 * body + comp6;
            double dv = act ? __ldcg(dvp) : 0.0;
            for (int c = c0; c < c0 + n; c++)
                for (int r = 0; r < 3; r++) {
                    double l = C.lam[r * ccap + c];
                    if (act) dv = fma(Mj[(12 * r + lane) * mcap + c], l, dv);
                }
            if (act) __stcg(dvp, dv);
        }
        if (!grid_barrier_f(dc, nblocks)) return;
    }
    int done = 0;
    double change = 0;
    for (int it = 0; it < iters; it++) {
        const int par = it & 1;
        const bool last = (it == iters - 1);
        double mx = 0;
        for (int col = 0; col < ncol; col++) {
            for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
                int g = groupOrder[k];
                int c0 = P.off[g], n = P.count[g];
                int body = act ? (side == 0 ? C.sb1[c0] : C.sb2[c0]) : 0;
                double* dvp = B.dv + 6 * body + comp6;
                double dv = act ? __ldcg(dvp) : 0.0;
                for (int c = c0; c < c0 + n; c++) {
                    double l0 = C.lam[c];
                    // normal row
                    {
                        double j = act ? C.J[lane * ccap + c] : 0.0;
                        double jd = hw_sum(j * dv, mask);
                        double nl = (C.bD[3 * ccap + c] * l0 - omega * (C.bD[c] + jd)) * invD[c];
                        nl = nl > 0.0 ? nl : 0.0;
                        double d = nl - l0;
                        if (act) dv = fma(Mj[lane * mcap + c], d, dv);
                        mx = fmax(mx, fabs(d));
                        l0 = nl;
                    }
                    double mu = mu_fast(B, C, c, fo, fv);
                    double lim = mu * l0;
                    for (int r = 1; r < 3; r++) {
                        double l = C.lam[r * ccap + c];
                        double j = act ? C.J[(12 * r + lane) * ccap + c] : 0.0;
                        double jd = hw_sum(j * dv, mask);
                        double nl = (C.bD[(3 + r) * ccap + c] * l - omega * (C.bD[r * ccap + c] + jd)) * invD[r * mcap + c];
                        nl = fmin(fmax(nl, -lim), lim);
                        double d = nl - l;
                        if (act) dv = fma(Mj[(12 * r + lane) * mcap + c], d, dv);
                        mx = fmax(mx, fabs(d));
                        if (lane == 0) C.lam[r * ccap + c] = nl;
                    }
                    if (lane == 0) C.lam[c] = l0;
                    if (last) {   // Contact.updateContactState
                        double j1 = act ? C.J[(12 + lane) * ccap + c] : 0.0;
                        double j2 = act ? C.J[(24 + lane) * ccap + c] : 0.0;
                        double w1 = C.bD[ccap + c] + hw_sum(j1 * dv, mask);
                        double w2 = C.bD[2 * ccap + c] + hw_sum(j2 * dv, mask);
                        int st;
                        if (fabs(l0) <= 1e-14) st = AM_STATE_BROKEN;
                        else if (fabs(w1) > slide) st = AM_STATE_ONEDGE;
                        else if (fabs(w2) > slide) st = AM_STATE_ONEDGE;
                        else st = AM_STATE_CLEAR;
                        if (lane == 0) C.state[c] = st;
                    }
                }
                if (act) __stcg(dvp, dv);
            }
            if (col == ncol - 1) {
                double wm = mx;
                for (int o = 16; o > 0; o >>= 1) wm = fmax(wm, __shfl_xor_sync(0xffffffffu, wm, o));
                if ((threadIdx.x & 31) == 0 && wm > 0)
                    atomicMax(&dc->maxchg[par], (unsigned long long)__double_as_longlong(wm));
            }
            if (!grid_barrier_f(dc, nblocks)) return;
        }
        change = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->maxchg[par]);
        done = it + 1;
        if (blockIdx.x == 0 && threadIdx.x == 0) dc->maxchg[par ^ 1] = 0ull;
        if (early && change < tol) break;
        if (check > 0 && resTol > 0 && (done % check == 0 || done == iters)) {
            // relative natural-map residual max|l - proj(l - w / (D + c))| / max(1, max|l|),
            // w = b + J dv + c l, over all contacts at the current state
            const int rp = (done / check) & 1;
            double rm = 0, lm = 0;
            for (int k = hw; k < colourOff[ncol]; k += nhw) {
                int g = groupOrder[k];
                int c0 = P.off[g], n = P.count[g];
                int body = act ? (side == 0 ? C.sb1[c0] : C.sb2[c0]) : 0;
                double dv = act ? __ldcg(B.dv + 6 * body + comp6) : 0.0;
                for (int c = c0; c < c0 + n; c++) {
                    double l0 = C.lam[c];
                    double lim = mu_fast(B, C, c, fo, fv) * l0;
                    for (int r = 0; r < 3; r++) {
                        double j = act ? C.J[(12 * r + lane) * ccap + c] : 0.0;
                        double jd = hw_sum(j * dv, mask);
                        double l = C.lam[r * ccap + c];
                        double w = C.bD[r * ccap + c] + jd + comp * l;
                        double z = l - w * invD[r * mcap + c];
                        z = r == 0 ? fmax(z, 0.0) : fmin(fmax(z, -lim), lim);
                        rm = fmax(rm, fabs(l - z));
                        lm = fmax(lm, fabs(l));
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                rm = fmax(rm, __shfl_xor_sync(0xffffffffu, rm, o));
                lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            }
            if ((threadIdx.x & 31) == 0) {
                if (rm > 0) atomicMax(&dc->reschk[rp], (unsigned long long)__double_as_longlong(rm));
                if (lm > 0) atomicMax(&dc->lamchk[rp], (unsigned long long)__double_as_longlong(lm));
            }
            if (!grid_barrier_f(dc, nblocks)) return;
            double res = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->reschk[rp]);
            double lmax = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->lamchk[rp]);
            if (blockIdx.x == 0 && threadIdx.x == 0) { dc->reschk[rp ^ 1] = 0ull; dc->lamchk[rp ^ 1] = 0ull; }
            if (res / fmax(1.0, lmax) <= resTol) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        dc->sweeps = done;
        dc->maxchg[0] = __double_as_longlong(change);
    }
}

const void* pgs_fast_kernel() { return (const void*)k_pgs_fast; }

void launch_pgs_fast(const DBodies& B, DContacts& C, DPairs& P, const int* groupOrder, const int* colourOff,
                     int ncol, int nc, int iters, double omega, double comp, double tol, bool early, int fo,
                     double fv, double slide, double* Mj, double* invD, int mcap, DCount* dc, int gridBlocks,
                     cudaStream_t s, double resTol, int check) {
    if (ncol <= 0 || nc <= 0) return;
    k_fast_prep<<<(nc + 127) / 128, 128, 0, s>>>(B, C, nc, comp, Mj, invD, mcap);
    AM_LAUNCHED(1);
    cudaMemsetAsync(&dc->maxchg, 0, sizeof(unsigned long long) * 2, s);
    cudaMemsetAsync(&dc->bar_count, 0, sizeof(int) * 2, s);
    cudaMemsetAsync(&dc->reschk, 0, sizeof(unsigned long long) * 4, s);
    int earlyI = early ? 1 : 0;
    DBodies Bc = B;
    void* args[] = {&Bc, &C, &P, (void*)&groupOrder, (void*)&colourOff, &ncol, &iters, &omega, &tol, &earlyI,
                    &fo, &fv, &slide, (void*)&Mj, (void*)&invD, &mcap, &dc, &comp, &resTol, &check};
    cudaLaunchCooperativeKernel((void*)k_pgs_fast, dim3(gridBlocks), dim3(128), args, 0, s);
    AM_LAUNCHED(1);
}

}  // namespace am
