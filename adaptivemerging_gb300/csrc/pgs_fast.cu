// pgs_fast.cu -- coloured projected Gauss-Seidel, FP64, latency-optimised.
//
// GB300 runs one FP64 warp instruction per 64 cycles per SM sub-partition,
// whatever the number of active lanes, and independent FP64 instructions do
// not overlap (measured: a chain of dependent DFMAs and four interleaved
// chains both cost 64 cycles per instruction; FP32 costs 4).  A Gauss-Seidel
// sweep in FP64 is therefore priced by the number of FP64 warp instructions
// on its critical path, not by HBM.  This kernel minimises that count:
//   * one 16-lane half-warp per body-pair group; lane k (k < 12) owns Jacobian
//     entry k of a row (a.v xyz, a.w xyz, b.v xyz, b.w xyz) and the matching
//     delta-v component, held in a register for the whole group (the group's
//     two bodies are touched by no other group of the same colour);
//   * the three rows' w = b + J . dv come from one interleaved shuffle
//     reduction (3 FMAs + 5 adds for all three rows, b folded in by lane 0);
//     the later rows of a contact follow the earlier rows' updates through
//     the precomputed couplings G_ij = J_i M^-1 J_j^T (PGS.java:140-178 makes
//     the same three row updates, each against the delta-v its predecessors
//     left), so the contact needs no second reduction;
//   * the projected update is lambda' = A l - q w with A = D / (D + c) and
//     q = omega / (D + c) precomputed per row; projections and the max-change
//     tracking compare IEEE bit patterns in the integer pipe;
//   * the next contact's operands are loaded while the current one computes.
// Contacts of a group stay sequential in list order; colours are separated
// by the bounded grid barrier.  Results equal the reference's fixed point,
// not its per-sweep bits (AM_ORDER_COLOURED); this translation unit is
// compiled with FMA contraction on.
#include <cuda_runtime.h>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"
#include "grid_sync.cuh"

namespace am {
using namespace amd;

// rows of the per-contact constant table K (stride cap)
enum : int { K_INVD = 0, K_A = 3, K_Q = 6, K_G10 = 9, K_G20 = 10, K_G21 = 11, K_MU = 12 };
int pgs_fast_krows() { return 13; }

__device__ __forceinline__ double mu_fast(const DBodies& B, const DContacts& C, int c, int fo, double fv) {
    if (fo) return fv;
    double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
    if (f1 < 0.2 || f2 < 0.2) return fmin(f1, f2);
    if (f1 > 1. || f2 > 1.) return fmax(f1, f2);
    return (f1 + f2) / 2.;
}

// per-contact precompute: Mj[36] (M^-1 J^T entries, row-major by row then
// lane k) and the constant table K: 1/(D + c), A, q per row, the couplings
// G10, G20, G21 and the contact's friction coefficient
__global__ void k_fast_prep(DBodies B, DContacts C, int nc, double comp, double omega, int fo, double fv,
                            double* Mj, double* K, int cap) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int ccap = C.cap;
    int s1 = C.sb1[c], s2 = C.sb2[c];
    double m1 = B.minv[s1], m2 = B.minv[s2];
    double mj[2][12];
    for (int r = 0; r < 3; r++) {
        double row[12];
        for (int k = 0; k < 3; k++) {
            row[k] = m1 * C.J[(12 * r + k) * ccap + c];          // a.v
            row[3 + k] = C.Ia[(3 * r + k) * ccap + c];           // jinv1 a.w
            row[6 + k] = m2 * C.J[(12 * r + 6 + k) * ccap + c];  // b.v
            row[9 + k] = C.Ib[(3 * r + k) * ccap + c];           // jinv2 b.w
        }
        for (int k = 0; k < 12; k++) Mj[(12 * r + k) * cap + c] = row[k];
        if (r < 2)
            for (int k = 0; k < 12; k++) mj[r][k] = row[k];
        double d = C.bD[(3 + r) * ccap + c];
        double inv = 1.0 / (d + comp);
        K[(K_INVD + r) * cap + c] = inv;
        K[(K_A + r) * cap + c] = d * inv;
        K[(K_Q + r) * cap + c] = omega * inv;
    }
    double g10 = 0, g20 = 0, g21 = 0;
    for (int k = 0; k < 12; k++) {
        double j1 = C.J[(12 + k) * ccap + c], j2 = C.J[(24 + k) * ccap + c];
        g10 = fma(j1, mj[0][k], g10);
        g20 = fma(j2, mj[0][k], g20);
        g21 = fma(j2, mj[1][k], g21);
    }
    K[K_G10 * cap + c] = g10;
    K[K_G20 * cap + c] = g20;
    K[K_G21 * cap + c] = g21;
    K[K_MU * cap + c] = mu_fast(B, C, c, fo, fv);
}

__device__ __forceinline__ double hw_sum(double v, unsigned mask) {
    v += __shfl_xor_sync(mask, v, 8, 16);
    v += __shfl_xor_sync(mask, v, 4, 16);
    v += __shfl_xor_sync(mask, v, 2, 16);
    v += __shfl_xor_sync(mask, v, 1, 16);
    return v;
}

// sums over the 16 lanes of a half-warp of p0, p1, p2 in five FP64 adds:
// the first level keeps rows 0 and 1 on lanes 0-7 and row 2 on lanes 8-15,
// the second keeps one row per quarter (rows 0, 1, 2, empty), the last two
// finish each quarter; the totals are then read from lanes 0, 4 and 8
__device__ __forceinline__ void hw_sum3(double p0, double p1, double p2, unsigned mask, int lane, double& s0,
                                        double& s1, double& s2) {
    const bool hi8 = (lane & 8) != 0, hi4 = (lane & 4) != 0;
    double a = (hi8 ? p2 : p0) + __shfl_xor_sync(mask, hi8 ? p0 : p2, 8, 16);
    double b = (hi8 ? 0.0 : p1) + __shfl_xor_sync(mask, hi8 ? p1 : 0.0, 8, 16);
    double t = (hi4 ? b : a) + __shfl_xor_sync(mask, hi4 ? a : b, 4, 16);
    t += __shfl_xor_sync(mask, t, 2, 16);
    t += __shfl_xor_sync(mask, t, 1, 16);
    s0 = __shfl_sync(mask, t, 0, 16);
    s1 = __shfl_sync(mask, t, 4, 16);
    s2 = __shfl_sync(mask, t, 8, 16);
}

// max(x, 0) (PGS.java:150) by the sign bit
__device__ __forceinline__ double pos_part(double x) { return __double_as_longlong(x) < 0 ? 0.0 : x; }

// clamp to [-lim, lim] (PGS.java:166-167), lim >= 0, by the magnitude bits
__device__ __forceinline__ double clamp_abs(double x, double lim) {
    long long xb = __double_as_longlong(x);
    long long lb = __double_as_longlong(lim);
    return (xb & 0x7fffffffffffffffll) > lb ? __longlong_as_double((xb & (long long)0x8000000000000000ull) | lb) : x;
}

__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// a contact's operands for one lane: its Jacobian and M^-1 J^T entries, and
// the per-contact scalars (every lane holds them)
struct FastOps {
    double j0, j1, j2, m0, m1, m2;
    double b0, b1, b2, l0, l1, l2;
    double a0, a1, a2, q0, q1, q2;
    double g10, g20, g21, mu;
};

__device__ __forceinline__ void load_ops(FastOps& o, const DContacts& C, const double* Mj, const double* K, int mcap,
                                         int c, int lane, bool act) {
    const int ccap = C.cap;
    o.j0 = act ? __ldg(C.J + lane * ccap + c) : 0.0;
    o.j1 = act ? __ldg(C.J + (12 + lane) * ccap + c) : 0.0;
    o.j2 = act ? __ldg(C.J + (24 + lane) * ccap + c) : 0.0;
    o.m0 = act ? __ldg(Mj + lane * mcap + c) : 0.0;
    o.m1 = act ? __ldg(Mj + (12 + lane) * mcap + c) : 0.0;
    o.m2 = act ? __ldg(Mj + (24 + lane) * mcap + c) : 0.0;
    o.b0 = __ldg(C.bD + c);
    o.b1 = __ldg(C.bD + ccap + c);
    o.b2 = __ldg(C.bD + 2 * ccap + c);
    o.l0 = __ldcg(C.lam + c);
    o.l1 = __ldcg(C.lam + ccap + c);
    o.l2 = __ldcg(C.lam + 2 * ccap + c);
    o.a0 = __ldg(K + K_A * mcap + c);
    o.a1 = __ldg(K + (K_A + 1) * mcap + c);
    o.a2 = __ldg(K + (K_A + 2) * mcap + c);
    o.q0 = __ldg(K + K_Q * mcap + c);
    o.q1 = __ldg(K + (K_Q + 1) * mcap + c);
    o.q2 = __ldg(K + (K_Q + 2) * mcap + c);
    o.g10 = __ldg(K + K_G10 * mcap + c);
    o.g20 = __ldg(K + K_G20 * mcap + c);
    o.g21 = __ldg(K + K_G21 * mcap + c);
    o.mu = __ldg(K + K_MU * mcap + c);
}

__global__ void __launch_bounds__(128) k_pgs_fast(DBodies B, DContacts C, DPairs P, const int* groupOrder,
                                                   const int* colourOff, int ncol, int iters, double tol, int early,
                                                   double slide, const double* Mj, const double* K, int mcap,
                                                   DCount* dc, double comp, double resTol, int check) {
    const int nblocks = gridDim.x;
    const int lane = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const unsigned mask = 0xFFFFu << (16 * half);
    const int hw = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    const int nhw = (nblocks * blockDim.x) >> 4;
    const int ccap = C.cap;
    const bool act = lane < 12;
    const bool lead = lane == 0;
    const int side = lane / 6;         // 0: body 1, 1: body 2
    const int comp6 = lane % 6;        // v xyz, w xyz
    unsigned target = 0;

    // confidentWarmStart (PGS.java:250-256), colour by colour
    for (int col = 0; col < ncol; col++) {
        for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
            int g = groupOrder[k];
            int c0 = P.off[g], n = P.count[g];
            int body = act ? (side == 0 ? C.sb1[c0] : C.sb2[c0]) : 0;
            double* dvp = B.dv + 6 * body + comp6;
            double dv = act ? __ldcg(dvp) : 0.0;
            for (int c = c0; c < c0 + n; c++)
                for (int r = 0; r < 3; r++) {
                    double l = __ldcg(C.lam + r * ccap + c);
                    if (act) dv = fma(__ldg(Mj + (12 * r + lane) * mcap + c), l, dv);
                }
            if (act) __stcg(dvp, dv);
        }
        if (!grid_barrier_counted(dc, nblocks, target)) return;
    }
    int done = 0;
    double change = 0;
    for (int it = 0; it < iters; it++) {
        const int par = it & 1;
        const bool last = (it == iters - 1);
        unsigned long long mx = 0;
        for (int col = 0; col < ncol; col++) {
            for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
                int g = groupOrder[k];
                int c0 = P.off[g], n = P.count[g];
                int body = act ? (side == 0 ? C.sb1[c0] : C.sb2[c0]) : 0;
                double* dvp = B.dv + 6 * body + comp6;
                double dv = act ? __ldcg(dvp) : 0.0;
                FastOps cur, nxt;
                load_ops(cur, C, Mj, K, mcap, c0, lane, act);
                for (int c = c0; c < c0 + n; c++) {
                    if (c + 1 < c0 + n) load_ops(nxt, C, Mj, K, mcap, c + 1, lane, act);
                    // w_r = b_r + J_r . dv for the three rows at once
                    double w0, w1, w2;
                    hw_sum3(fma(cur.j0, dv, lead ? cur.b0 : 0.0), fma(cur.j1, dv, lead ? cur.b1 : 0.0),
                            fma(cur.j2, dv, lead ? cur.b2 : 0.0), mask, lane, w0, w1, w2);
                    // normal row, then the two friction rows inside mu * lambda_n
                    double n0 = pos_part(fma(-cur.q0, w0, cur.a0 * cur.l0));
                    double d0 = n0 - cur.l0;
                    double lim = cur.mu * n0;
                    w1 = fma(cur.g10, d0, w1);
                    w2 = fma(cur.g20, d0, w2);
                    double n1 = clamp_abs(fma(-cur.q1, w1, cur.a1 * cur.l1), lim);
                    double d1 = n1 - cur.l1;
                    w2 = fma(cur.g21, d1, w2);
                    double n2 = clamp_abs(fma(-cur.q2, w2, cur.a2 * cur.l2), lim);
                    double d2 = n2 - cur.l2;
                    dv = fma(cur.m0, d0, dv);
                    dv = fma(cur.m1, d1, dv);
                    dv = fma(cur.m2, d2, dv);
                    mx = max(mx, max(abs_bits(d0), max(abs_bits(d1), abs_bits(d2))));
                    if (lead) {
                        C.lam[c] = n0;
                        C.lam[ccap + c] = n1;
                        C.lam[2 * ccap + c] = n2;
                    }
                    if (last) {   // Contact.updateContactState, at the contact's final delta-v
                        double u0, u1, u2;
                        hw_sum3(0.0, fma(cur.j1, dv, lead ? cur.b1 : 0.0), fma(cur.j2, dv, lead ? cur.b2 : 0.0),
                                mask, lane, u0, u1, u2);
                        int st;
                        if (fabs(n0) <= 1e-14) st = AM_STATE_BROKEN;
                        else if (fabs(u1) > slide) st = AM_STATE_ONEDGE;
                        else if (fabs(u2) > slide) st = AM_STATE_ONEDGE;
                        else st = AM_STATE_CLEAR;
                        if (lead) C.state[c] = st;
                    }
                    cur = nxt;
                }
                if (act) __stcg(dvp, dv);
            }
            if (col == ncol - 1) {
                unsigned long long wm = mx;
                for (int o = 16; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
                if ((threadIdx.x & 31) == 0 && wm > 0) atomicMax(&dc->maxchg[par], wm);
            }
            if (!grid_barrier_counted(dc, nblocks, target)) return;
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
                    double l0 = __ldcg(C.lam + c);
                    double lim = __ldg(K + K_MU * mcap + c) * l0;
                    for (int r = 0; r < 3; r++) {
                        double j = act ? __ldg(C.J + (12 * r + lane) * ccap + c) : 0.0;
                        double jd = hw_sum(j * dv, mask);
                        double l = __ldcg(C.lam + r * ccap + c);
                        double w = C.bD[r * ccap + c] + jd + comp * l;
                        double z = l - w * __ldg(K + (K_INVD + r) * mcap + c);
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
            if (!grid_barrier_counted(dc, nblocks, target)) return;
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
                     double fv, double slide, double* Mj, double* K, int mcap, DCount* dc, int gridBlocks,
                     cudaStream_t s, double resTol, int check) {
    if (ncol <= 0 || nc <= 0) return;
    k_fast_prep<<<(nc + 127) / 128, 128, 0, s>>>(B, C, nc, comp, omega, fo, fv, Mj, K, mcap);
    AM_LAUNCHED(1);
    cudaMemsetAsync(&dc->maxchg, 0, sizeof(unsigned long long) * 2, s);
    cudaMemsetAsync(&dc->bar_count, 0, sizeof(int), s);
    cudaMemsetAsync(&dc->reschk, 0, sizeof(unsigned long long) * 4, s);
    int earlyI = early ? 1 : 0;
    DBodies Bc = B;
    const double* Mjc = Mj;
    const double* Kc = K;
    void* args[] = {&Bc, &C, &P, (void*)&groupOrder, (void*)&colourOff, &ncol, &iters, &tol, &earlyI,
                    &slide, (void*)&Mjc, (void*)&Kc, &mcap, &dc, &comp, &resTol, &check};
    cudaLaunchCooperativeKernel((void*)k_pgs_fast, dim3(gridBlocks), dim3(128), args, 0, s);
    AM_LAUNCHED(1);
}

}  // namespace am
