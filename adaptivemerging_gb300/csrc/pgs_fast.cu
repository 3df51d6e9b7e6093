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
__device__ __forceinline__ void fast_prep_contact(const DBodies& B, const DContacts& C, int c, double comp,
                                                  double omega, int fo, double fv, double* Mj, double* K, int cap) {
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

__global__ void k_fast_prep(DBodies B, DContacts C, int nc, double comp, double omega, int fo, double fv,
                            double* Mj, double* K, int cap) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    fast_prep_contact(B, C, c, comp, omega, fo, fv, Mj, K, cap);
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
        const int par = it % 3;
        if (blockIdx.x == 0 && threadIdx.x == 0) dc->maxchg[(it + 1) % 3] = 0ull;   // the next sweep's slot
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
    cudaMemsetAsync(&dc->maxchg, 0, sizeof(dc->maxchg), s);
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

// ---------------------------------------------------------------------------
// AM_ORDER_MIXED: the same coloured Gauss-Seidel, its sweeps in FP32 on the
// correction to an FP64 base, refined in FP64 every few sweeps.
//
// At a base point (lambda0, dv0 = M^-1 J^T lambda0, both FP64) every contact
// row gets, in FP64, r = b + J dv0 and the constant of its projected update
//   s = (A - 1) lambda0 - q r,
// so that lambda0 + mu updates as mu' = P(s + A mu - q (J u)) with u the
// delta-v correction M^-1 J^T mu; P shifts the bounds by lambda0:
//   normal   mu_n' >= -lambda0_n
//   friction f - mu_c mu_n' <= mu_t' <= e + mu_c mu_n',
//            e = mu_c lambda0_n - lambda0_t,  f = -mu_c lambda0_n - lambda0_t.
// The sweeps update mu and u in FP32.  Every constant above vanishes at the
// fixed point (s for a row inside its bounds, e or f for a row at one), and
// mu and u are corrections that shrink with the iteration, so FP32 keeps its
// relative precision on what is left to solve.  A refinement folds
// lambda = P64(lambda0 + mu) in FP64 and carries dv along with the exact
// FP64 differences (colour by colour, as the sweep does), then takes a new
// base point.  This is iterative refinement of the projected Gauss-Seidel
// fixed point (the FP32 sweep is the inner solver, the FP64 base the outer
// residual), so the converged multipliers are the FP64 iteration's.  On
// GB300 an FP32 warp instruction issues in a cycle and completes in about
// four, where an FP64 one occupies its pipe for 64 cycles: the sweep's
// dependent chain, which bounds a single scene, is about ten times shorter.
// ---------------------------------------------------------------------------

// The FP32 sweep runs one thread per body-pair group (the group's two bodies'
// corrections u stay in registers across its contacts).  Per contact it
// evaluates J_q u = f_q . (u_b.v - u_a.v) + ja_q . u_a.w + jb_q . u_b.w for
// the three rows from its own Jacobian entries (f_q the row's b.v part, which
// is minus its a.v part; ja_q and jb_q the angular parts), and applies the
// impulse through the solve bodies' inverse mass and world inverse inertia:
// the same M^-1 J^T as the FP64 passes, rounded to FP32.
//
// Per contact, MIX_REC floats (12 float4): the Jacobian and solve constants
// (9 float4, written by k_mixed_pack), the base constants (2 float4, written
// at every base point) and the corrections with the friction coefficient
// (1 float4).  Per body, 8 floats: minv and the symmetric part of jinv.
enum : int {
    R_F = 0, R_JA = 9, R_JB = 18, R_G10 = 27, R_G20 = 28, R_G21 = 29, R_QQ = 30, R_A = 33,
    R_S = 36, R_LO = 39, R_E1 = 40, R_F1 = 41, R_E2 = 42, R_F2 = 43, R_M = 44, R_MU = 47, MIX_REC = 48
};
int pgs_mixed_frows() { return MIX_REC; }

__device__ __forceinline__ void mixed_pack_contact(const DContacts& C, int c, const double* K, float* F, int cap) {
    const int ccap = C.cap;
    float r[MIX_REC];
    for (int q = 0; q < 3; q++)
        for (int k = 0; k < 3; k++) {
            r[R_F + 3 * q + k] = (float)C.J[(12 * q + 6 + k) * ccap + c];
            r[R_JA + 3 * q + k] = (float)C.J[(12 * q + 3 + k) * ccap + c];
            r[R_JB + 3 * q + k] = (float)C.J[(12 * q + 9 + k) * ccap + c];
        }
    r[R_G10] = (float)K[K_G10 * cap + c];
    r[R_G20] = (float)K[K_G20 * cap + c];
    r[R_G21] = (float)K[K_G21 * cap + c];
    for (int q = 0; q < 3; q++) {
        r[R_QQ + q] = (float)K[(K_Q + q) * cap + c];
        r[R_A + q] = (float)K[(K_A + q) * cap + c];
    }
    for (int k = R_S; k < R_MU; k++) r[k] = 0.f;
    r[R_MU] = (float)K[K_MU * cap + c];
    float4* dst = reinterpret_cast<float4*>(F + (size_t)MIX_REC * c);
    for (int k = 0; k < MIX_REC / 4; k++) dst[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
}

// the FP64 constants (as k_fast_prep) and the FP32 record of a contact
__global__ void k_mixed_prep(DBodies B, DContacts C, int nc, double comp, double omega, int fo, double fv,
                             double* Mj, double* K, float* F, int cap) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    fast_prep_contact(B, C, c, comp, omega, fo, fv, Mj, K, cap);
    mixed_pack_contact(C, c, K, F, cap);
}

// the coloured groups in sweep order, flattened: first contact, contact
// count and the two solve bodies (bit 31 set for a pinned body), so that a
// sweep reads one record per group instead of a chain of four indirections
// ... and per body (b < nb) its FP32 inverse mass and the symmetric part of
// its world inverse inertia
__global__ void k_mixed_groups(DBodies B, DContacts C, DPairs P, const int* groupOrder, int ng, int4* GI, int nb,
                               float* BM) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nb) {
        const double* J = B.jinv + 9 * (size_t)k;
        float4* d = reinterpret_cast<float4*>(BM + 8 * (size_t)k);
        d[0] = make_float4((float)B.minv[k], (float)J[0], (float)J[4], (float)J[8]);
        d[1] = make_float4((float)J[1], (float)J[2], (float)J[5], 0.f);
    }
    if (k >= ng) return;
    const int g = groupOrder[k];
    const int c0 = P.off[g];
    const int sa = C.sb1[c0], sb = C.sb2[c0];
    const int pa = (B.flags[sa] & F_PINNED) ? (int)0x80000000u : 0, pb = (B.flags[sb] & F_PINNED) ? (int)0x80000000u : 0;
    GI[k] = make_int4(c0, P.count[g], sa | pa, sb | pb);
}

// Storage modes of the mixed solve: 0, a cooperative grid (values the kernel
// writes and reads back go through L2); 1, one block with the contact
// records in global memory (the block sees its own stores through L1 after
// __syncthreads, so it loads them plainly) and the body data in shared
// memory; 2, one block with the contact records in shared memory too.
template <bool ONE> __device__ __forceinline__ float4 ldw4(const float4* p) { return ONE ? *p : __ldcg(p); }
template <bool ONE> __device__ __forceinline__ void stw4(float4* p, float4 v) {
    if (ONE) *p = v;
    else __stcg(p, v);
}
template <bool ONE> __device__ __forceinline__ float ldw(const float* p) { return ONE ? *p : __ldcg(p); }
template <bool ONE> __device__ __forceinline__ void stw(float* p, float v) {
    if (ONE) *p = v;
    else __stcg(p, v);
}
template <bool ONE> __device__ __forceinline__ double ldw(const double* p) { return ONE ? *p : __ldcg(p); }
template <bool ONE> __device__ __forceinline__ void stw(double* p, double v) {
    if (ONE) *p = v;
    else __stcg(p, v);
}
// read-only records: shared memory (mode 2) or the read-only path
template <int MODE> __device__ __forceinline__ float4 ldr4(const float4* p) { return MODE == 2 ? *p : __ldg(p); }
// read-only body data: shared memory (one block) or the read-only path
template <bool ONE> __device__ __forceinline__ float4 ldb4(const float4* p) { return ONE ? *p : __ldg(p); }
template <bool ONE> __device__ __forceinline__ bool mixed_bar(DCount* dc, int nblocks, unsigned& target) {
    if (ONE) {   // nothing else can raise an error inside a one-block solve
        __syncthreads();
        return true;
    }
    return grid_barrier_counted(dc, nblocks, target);
}

// one contact's FP32 operands; t = s + A mu is formed at load time (off the
// dependent chain)
struct MixRec {
    float f[9], ja[9], jb[9];
    float g10, g20, g21, qq[3];
    float t[3], lo, e1, f1, e2, f2, m[3], mu;
};

template <int MODE>
__device__ __forceinline__ void load_mixrec(MixRec& o, const float* F, int c) {
    constexpr bool ONE = MODE > 0;
    const float4* p = reinterpret_cast<const float4*>(F + (size_t)MIX_REC * c);
    float r[36];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        float4 v = ldr4<MODE>(p + k);
        r[4 * k] = v.x; r[4 * k + 1] = v.y; r[4 * k + 2] = v.z; r[4 * k + 3] = v.w;
    }
    const float4 s0 = ldw4<ONE>(p + 9), s1 = ldw4<ONE>(p + 10), m = ldw4<ONE>(p + 11);
#pragma unroll
    for (int k = 0; k < 9; k++) { o.f[k] = r[R_F + k]; o.ja[k] = r[R_JA + k]; o.jb[k] = r[R_JB + k]; }
    o.g10 = r[R_G10]; o.g20 = r[R_G20]; o.g21 = r[R_G21];
    o.qq[0] = r[R_QQ]; o.qq[1] = r[R_QQ + 1]; o.qq[2] = r[R_QQ + 2];
    o.m[0] = m.x; o.m[1] = m.y; o.m[2] = m.z; o.mu = m.w;
    o.t[0] = fmaf(r[R_A], m.x, s0.x);
    o.t[1] = fmaf(r[R_A + 1], m.y, s0.y);
    o.t[2] = fmaf(r[R_A + 2], m.z, s0.z);
    o.lo = s0.w; o.e1 = s1.x; o.f1 = s1.y; o.e2 = s1.z; o.f2 = s1.w;
}

// o += symmetric matrix (xx yy zz xy xz yz) times v
__device__ __forceinline__ void symv_add(const float* m, const float* v, float* o) {
    o[0] = fmaf(m[4], v[2], fmaf(m[3], v[1], fmaf(m[0], v[0], o[0])));
    o[1] = fmaf(m[5], v[2], fmaf(m[1], v[1], fmaf(m[3], v[0], o[1])));
    o[2] = fmaf(m[2], v[2], fmaf(m[5], v[1], fmaf(m[4], v[0], o[2])));
}

// MODE 1 and 2: a single block of NT threads solves the scene; its barriers
// are block barriers, the body data and delta-v corrections live in shared
// memory (mode 2 adds the contact records) and the sweep maxima in shared
// words.  MODE 0: a cooperative grid of NT-thread blocks with the bounded
// grid barrier.  The FP64 passes run a 16-lane half-warp per group or
// contact, as the FP64 kernel does; the FP32 sweep a thread per group.
template <int MODE, int NT>
__global__ void __launch_bounds__(NT) k_pgs_mixed(DBodies B, DContacts C, DPairs P,
                                                   const int* colourOffG, const int4* GIg, int ncol, int nc,
                                                   int nbodies, int iters, double tol, int early, double slide,
                                                   const double* Mj, const double* K, float* Fg, float* BMg,
                                                   float* Ug, int mcap, int refine, DCount* dc, double comp,
                                                   double resTol, int check) {
    constexpr bool ONE = MODE > 0;
    extern __shared__ float4 s_dyn4[];
    __shared__ unsigned s_mx[3];
    __shared__ unsigned long long s_res[2], s_lam[2];
    float* s_dyn = reinterpret_cast<float*>(s_dyn4);
    // shared layout (one block): body data (8 floats a body), corrections (6
    // floats a body, padded to 8), the group records (4 ints a group), the
    // colour offsets (padded to 4 ints), then in mode 2 the contact records
    const int ng = ncol > 0 ? colourOffG[ncol] : 0;
    const size_t oGI = 16 * (size_t)nbodies, oCO = oGI + 4 * (size_t)ng, oF = oCO + ((ncol + 4) & ~3);
    float* BM = ONE ? s_dyn : BMg;
    float* U = ONE ? s_dyn + 8 * (size_t)nbodies : Ug;
    const int4* GI = ONE ? reinterpret_cast<const int4*>(s_dyn + oGI) : GIg;
    const int* colourOff = ONE ? reinterpret_cast<const int*>(s_dyn + oCO) : colourOffG;
    float* F = MODE == 2 ? s_dyn + oF : Fg;
    const int nblocks = ONE ? 1 : gridDim.x;
    const int tid = blockIdx.x * NT + threadIdx.x, nthr = nblocks * NT;
    const int lane = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const unsigned mask = 0xFFFFu << (16 * half);
    const int hw = tid >> 4, nhw = nthr >> 4;
    const int ccap = C.cap;
    const bool act = lane < 12;
    const bool lead = lane == 0;
    const int side = lane / 6;
    const int comp6 = lane % 6;
    const bool wantRes = check > 0 && resTol > 0;
    unsigned target = 0;
    if (ONE) {
        if (threadIdx.x < 3) s_mx[threadIdx.x] = 0u;
        if (threadIdx.x < 2) { s_res[threadIdx.x] = 0ull; s_lam[threadIdx.x] = 0ull; }
        const float4* src = reinterpret_cast<const float4*>(BMg);
        for (int i = threadIdx.x; i < 2 * nbodies; i += NT) s_dyn4[i] = __ldg(src + i);
        int4* gi = reinterpret_cast<int4*>(s_dyn + oGI);
        for (int i = threadIdx.x; i < ng; i += NT) gi[i] = __ldg(GIg + i);
        int* co = reinterpret_cast<int*>(s_dyn + oCO);
        for (int i = threadIdx.x; i <= ncol; i += NT) co[i] = __ldg(colourOffG + i);
        if (MODE == 2) {
            float4* dst = reinterpret_cast<float4*>(F);
            const float4* fs = reinterpret_cast<const float4*>(Fg);
            for (int i = threadIdx.x; i < (MIX_REC / 4) * nc; i += NT) dst[i] = __ldg(fs + i);
        }
        __syncthreads();   // the copies are read from here on
    }

    // confidentWarmStart (PGS.java:250-256), colour by colour, FP64
    for (int col = 0; col < ncol; col++) {
        for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
            const int4 gi = ONE ? GI[k] : __ldg(GI + k);
            const int c0 = gi.x, n = gi.y;
            int body = act ? (side == 0 ? gi.z : gi.w) & 0x7fffffff : 0;
            double* dvp = B.dv + 6 * body + comp6;
            double dv = act ? ldw<ONE>(dvp) : 0.0;
            for (int c = c0; c < c0 + n; c++)
                for (int r = 0; r < 3; r++) {
                    double l = ldw<ONE>(C.lam + r * ccap + c);
                    if (act) dv = fma(__ldg(Mj + (12 * r + lane) * mcap + c), l, dv);
                }
            if (act) stw<ONE>(dvp, dv);
        }
        if (!mixed_bar<ONE>(dc, nblocks, target)) return;
    }

    // a new FP64 base point at the current (lambda, dv): the FP32 constants,
    // corrections reset to zero, the natural-map residual (slot rp, when a
    // residual target is set) and the contact states
    // (Contact.updateContactState at this delta-v)
    auto base = [&](int rp) -> bool {
        for (int i = tid; i < 6 * nbodies; i += nthr) stw<ONE>(U + i, 0.f);
        double rm = 0, lm = 0;
        for (int c = hw; c < nc; c += nhw) {
            int body = act ? (side == 0 ? C.sb1[c] : C.sb2[c]) : 0;
            double dv = act ? ldw<ONE>(B.dv + 6 * body + comp6) : 0.0;
            double j0 = act ? __ldg(C.J + lane * ccap + c) : 0.0;
            double j1 = act ? __ldg(C.J + (12 + lane) * ccap + c) : 0.0;
            double j2 = act ? __ldg(C.J + (24 + lane) * ccap + c) : 0.0;
            double r0, r1, r2;
            hw_sum3(fma(j0, dv, lead ? __ldg(C.bD + c) : 0.0), fma(j1, dv, lead ? __ldg(C.bD + ccap + c) : 0.0),
                    fma(j2, dv, lead ? __ldg(C.bD + 2 * ccap + c) : 0.0), mask, lane, r0, r1, r2);
            const double l0 = ldw<ONE>(C.lam + c), l1 = ldw<ONE>(C.lam + ccap + c);
            const double l2 = ldw<ONE>(C.lam + 2 * ccap + c);
            const double lim = __ldg(K + K_MU * mcap + c) * l0;
            if (wantRes) {
                double z0 = fmax(l0 - (r0 + comp * l0) * __ldg(K + K_INVD * mcap + c), 0.0);
                double z1 = fmin(fmax(l1 - (r1 + comp * l1) * __ldg(K + (K_INVD + 1) * mcap + c), -lim), lim);
                double z2 = fmin(fmax(l2 - (r2 + comp * l2) * __ldg(K + (K_INVD + 2) * mcap + c), -lim), lim);
                rm = fmax(rm, fmax(fabs(l0 - z0), fmax(fabs(l1 - z1), fabs(l2 - z2))));
                lm = fmax(lm, fmax(fabs(l0), fmax(fabs(l1), fabs(l2))));
            }
            if (lead) {
                float4* rec = reinterpret_cast<float4*>(F + (size_t)MIX_REC * c);
                const double s0 = (__ldg(K + K_A * mcap + c) - 1.0) * l0 - __ldg(K + K_Q * mcap + c) * r0;
                const double s1 = (__ldg(K + (K_A + 1) * mcap + c) - 1.0) * l1 - __ldg(K + (K_Q + 1) * mcap + c) * r1;
                const double s2 = (__ldg(K + (K_A + 2) * mcap + c) - 1.0) * l2 - __ldg(K + (K_Q + 2) * mcap + c) * r2;
                stw4<ONE>(rec + 9, make_float4((float)s0, (float)s1, (float)s2, (float)(-l0)));
                stw4<ONE>(rec + 10, make_float4((float)(lim - l1), (float)(-lim - l1), (float)(lim - l2),
                                                (float)(-lim - l2)));
                stw<ONE>(F + (size_t)MIX_REC * c + R_M, 0.f);
                stw<ONE>(F + (size_t)MIX_REC * c + R_M + 1, 0.f);
                stw<ONE>(F + (size_t)MIX_REC * c + R_M + 2, 0.f);
                int st;
                if (fabs(l0) <= 1e-14) st = AM_STATE_BROKEN;
                else if (fabs(r1) > slide) st = AM_STATE_ONEDGE;
                else if (fabs(r2) > slide) st = AM_STATE_ONEDGE;
                else st = AM_STATE_CLEAR;
                C.state[c] = st;
            }
        }
        if (wantRes) {
            for (int o = 16; o > 0; o >>= 1) {
                rm = fmax(rm, __shfl_xor_sync(0xffffffffu, rm, o));
                lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            }
            if ((threadIdx.x & 31) == 0) {
                unsigned long long* R = ONE ? s_res : dc->reschk;
                unsigned long long* L = ONE ? s_lam : dc->lamchk;
                if (rm > 0) atomicMax(R + rp, (unsigned long long)__double_as_longlong(rm));
                if (lm > 0) atomicMax(L + rp, (unsigned long long)__double_as_longlong(lm));
            }
        }
        return mixed_bar<ONE>(dc, nblocks, target);
    };

    // lambda = P64(lambda0 + mu), dv += M^-1 J^T (lambda - lambda0), colour by colour
    auto fold = [&]() -> bool {
        for (int col = 0; col < ncol; col++) {
            for (int k = colourOff[col] + hw; k < colourOff[col + 1]; k += nhw) {
                const int4 gi = ONE ? GI[k] : __ldg(GI + k);
                const int c0 = gi.x, n = gi.y;
                int body = act ? (side == 0 ? gi.z : gi.w) & 0x7fffffff : 0;
                double* dvp = B.dv + 6 * body + comp6;
                double dv = act ? ldw<ONE>(dvp) : 0.0;
                for (int c = c0; c < c0 + n; c++) {
                    const double l0 = ldw<ONE>(C.lam + c), l1 = ldw<ONE>(C.lam + ccap + c);
                    const double l2 = ldw<ONE>(C.lam + 2 * ccap + c);
                    const float* mp = F + (size_t)MIX_REC * c + R_M;
                    double n0 = pos_part(l0 + (double)ldw<ONE>(mp));
                    double lim = __ldg(K + K_MU * mcap + c) * n0;
                    double n1 = clamp_abs(l1 + (double)ldw<ONE>(mp + 1), lim);
                    double n2 = clamp_abs(l2 + (double)ldw<ONE>(mp + 2), lim);
                    if (act) {
                        dv = fma(__ldg(Mj + lane * mcap + c), n0 - l0, dv);
                        dv = fma(__ldg(Mj + (12 + lane) * mcap + c), n1 - l1, dv);
                        dv = fma(__ldg(Mj + (24 + lane) * mcap + c), n2 - l2, dv);
                    }
                    if (lead) {
                        stw<ONE>(C.lam + c, n0);
                        stw<ONE>(C.lam + ccap + c, n1);
                        stw<ONE>(C.lam + 2 * ccap + c, n2);
                    }
                }
                if (act) stw<ONE>(dvp, dv);
            }
            if (!mixed_bar<ONE>(dc, nblocks, target)) return false;
        }
        return true;
    };

    int nbase = 0;
    if (!base(nbase++ & 1)) return;
    int done = 0;
    double change = 0;
    for (int it = 0; it < iters; it++) {
        const int par = it % 3;
        if (blockIdx.x == 0 && threadIdx.x == 0) {   // the next sweep's slot
            if (ONE) s_mx[(it + 1) % 3] = 0u;
            else dc->maxchg[(it + 1) % 3] = 0ull;
        }
        const bool last = (it == iters - 1);
        float mx = 0.f;
        for (int col = 0; col < ncol; col++) {
            for (int k = colourOff[col] + tid; k < colourOff[col + 1]; k += nthr) {
                const int4 gi = ONE ? GI[k] : __ldg(GI + k);
                const int c0 = gi.x, n = gi.y;
                const int sa = gi.z & 0x7fffffff, sb = gi.w & 0x7fffffff;
                float ja[6], jb[6], ua[6], ub[6];
                const float4 a0 = ldb4<ONE>(reinterpret_cast<const float4*>(BM) + 2 * sa);
                const float4 a1 = ldb4<ONE>(reinterpret_cast<const float4*>(BM) + 2 * sa + 1);
                const float4 b0 = ldb4<ONE>(reinterpret_cast<const float4*>(BM) + 2 * sb);
                const float4 b1 = ldb4<ONE>(reinterpret_cast<const float4*>(BM) + 2 * sb + 1);
                const float ma = a0.x, mb = b0.x;
                ja[0] = a0.y; ja[1] = a0.z; ja[2] = a0.w; ja[3] = a1.x; ja[4] = a1.y; ja[5] = a1.z;
                jb[0] = b0.y; jb[1] = b0.z; jb[2] = b0.w; jb[3] = b1.x; jb[4] = b1.y; jb[5] = b1.z;
#pragma unroll
                for (int q = 0; q < 6; q++) { ua[q] = ldw<ONE>(U + 6 * sa + q); ub[q] = ldw<ONE>(U + 6 * sb + q); }
                // one contact's update; the records alternate between two
                // buffers (the next one loads while this one computes)
                auto update = [&](const MixRec& cur, int c) {
                    const float dvv[3] = {ub[0] - ua[0], ub[1] - ua[1], ub[2] - ua[2]};
                    float p[3];
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        const float x = fmaf(cur.f[3 * q + 2], dvv[2], fmaf(cur.f[3 * q + 1], dvv[1], cur.f[3 * q] * dvv[0]));
                        const float y = fmaf(cur.ja[3 * q + 2], ua[5], fmaf(cur.ja[3 * q + 1], ua[4], cur.ja[3 * q] * ua[3]));
                        const float z = fmaf(cur.jb[3 * q + 2], ub[5], fmaf(cur.jb[3 * q + 1], ub[4], cur.jb[3 * q] * ub[3]));
                        p[q] = x + (y + z);
                    }
                    const float n0 = fmaxf(fmaf(-cur.qq[0], p[0], cur.t[0]), cur.lo);
                    const float d0 = n0 - cur.m[0];
                    const float n1 = fminf(fmaxf(fmaf(-cur.qq[1], fmaf(cur.g10, d0, p[1]), cur.t[1]),
                                                 fmaf(-cur.mu, n0, cur.f1)),
                                           fmaf(cur.mu, n0, cur.e1));
                    const float d1 = n1 - cur.m[1];
                    const float n2 = fminf(fmaxf(fmaf(-cur.qq[2], fmaf(cur.g21, d1, fmaf(cur.g20, d0, p[2])), cur.t[2]),
                                                 fmaf(-cur.mu, n0, cur.f2)),
                                           fmaf(cur.mu, n0, cur.e2));
                    const float d2 = n2 - cur.m[2];
                    float Fi[3], Aa[3], Ab[3];
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        Fi[k] = fmaf(d2, cur.f[6 + k], fmaf(d1, cur.f[3 + k], d0 * cur.f[k]));
                        Aa[k] = fmaf(d2, cur.ja[6 + k], fmaf(d1, cur.ja[3 + k], d0 * cur.ja[k]));
                        Ab[k] = fmaf(d2, cur.jb[6 + k], fmaf(d1, cur.jb[3 + k], d0 * cur.jb[k]));
                    }
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        ua[k] = fmaf(-ma, Fi[k], ua[k]);
                        ub[k] = fmaf(mb, Fi[k], ub[k]);
                    }
                    symv_add(ja, Aa, ua + 3);
                    symv_add(jb, Ab, ub + 3);
                    mx = fmaxf(mx, fmaxf(fabsf(d0), fmaxf(fabsf(d1), fabsf(d2))));
                    stw4<ONE>(reinterpret_cast<float4*>(F + (size_t)MIX_REC * c + R_M), make_float4(n0, n1, n2, cur.mu));
                };
                MixRec r0, r1;
                const int c1 = c0 + n;
                load_mixrec<MODE>(r0, F, c0);
                for (int c = c0; c < c1; c += 2) {
                    if (c + 1 < c1) load_mixrec<MODE>(r1, F, c + 1);
                    update(r0, c);
                    if (c + 1 >= c1) break;
                    if (c + 2 < c1) load_mixrec<MODE>(r0, F, c + 2);
                    update(r1, c + 1);
                }
                // a pinned body's corrections stay zero (its inverse mass and
                // inertia are zero); groups of one colour may share it
                if (gi.z >= 0)
#pragma unroll
                    for (int q = 0; q < 6; q++) stw<ONE>(U + 6 * sa + q, ua[q]);
                if (gi.w >= 0)
#pragma unroll
                    for (int q = 0; q < 6; q++) stw<ONE>(U + 6 * sb + q, ub[q]);
            }
            if (col == ncol - 1) {
                unsigned wm = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));   // mx >= 0: bits order as values
                if ((threadIdx.x & 31) == 0 && wm > 0) {
                    if (ONE) atomicMax(&s_mx[par], wm);
                    else atomicMax(&dc->maxchg[par], (unsigned long long)__double_as_longlong((double)__uint_as_float(wm)));
                }
            }
            if (!mixed_bar<ONE>(dc, nblocks, target)) return;
        }
        if (ONE) change = (double)__uint_as_float(s_mx[par]);
        else change = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->maxchg[par]);
        done = it + 1;
        const bool stop = early && change < tol;
        const bool checkNow = wantRes && (done % check == 0 || last);
        if (!(last || stop || checkNow || (refine > 0 && done % refine == 0))) continue;
        if (!fold()) return;
        const int rp = nbase++ & 1;
        if (!base(rp)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (ONE) { s_res[rp ^ 1] = 0ull; s_lam[rp ^ 1] = 0ull; }
            else { dc->reschk[rp ^ 1] = 0ull; dc->lamchk[rp ^ 1] = 0ull; }
        }
        if (stop) break;
        if (checkNow) {
            double res, lmax;
            if (ONE) {
                res = __longlong_as_double((long long)s_res[rp]);
                lmax = __longlong_as_double((long long)s_lam[rp]);
            } else {
                res = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->reschk[rp]);
                lmax = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->lamchk[rp]);
            }
            if (res / fmax(1.0, lmax) <= resTol) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        dc->sweeps = done;
        dc->maxchg[0] = __double_as_longlong(change);
    }
}

static const int MIXED_GRID_NT = 128, MIXED_ONE_NT = 256;
static const int MIXED_SMEM_MAX = 220 * 1024;

const void* pgs_mixed_kernel() { return (const void*)k_pgs_mixed<0, MIXED_GRID_NT>; }

// dynamic shared memory of the one-block forms (4-byte words): body data and
// corrections, 16 a body; group records, 4 a group; colour offsets; mode 2
// adds the contact records
static size_t mixed_smem(int mode, int nc, int nbodies, int ng, int ncol) {
    return 4 * (16 * (size_t)nbodies + 4 * (size_t)ng + ((ncol + 4) & ~3) + (mode == 2 ? (size_t)MIX_REC * nc : 0));
}

int pgs_mixed_grid_blocks(int widest, int coopBlocks) {
    return std::min(coopBlocks, std::max(1, (widest + MIXED_GRID_NT - 1) / MIXED_GRID_NT));
}

bool pgs_mixed_fits(int mode, const std::vector<int>& colOff, int nbodies, int nc) {
    if (mode == 0) return true;
    const int ncol = (int)colOff.size() - 1, ng = ncol > 0 ? colOff[ncol] : 0;
    return mixed_smem(mode, nc, nbodies, ng, ncol) <= (size_t)MIXED_SMEM_MAX;
}

int pgs_mixed_mode(const std::vector<int>& colOff, int gridBlocks, int nbodies, int nc) {
    const int ncol = (int)colOff.size() - 1, ng = ncol > 0 ? colOff[ncol] : 0;
    if (mixed_smem(1, nc, nbodies, ng, ncol) > (size_t)MIXED_SMEM_MAX) return 0;
    // in half-passes (one pass: every thread runs one group's chain): a
    // colour costs its passes over the groups, and on a grid of several
    // blocks half a pass more for the grid barrier (on a 40 x 25 brick wall,
    // whose colours need two passes of one block, the grid form was 1.8 times
    // faster; on a merged wall of about 140 colours, one block was faster)
    const int tOne = MIXED_ONE_NT, tGrid = gridBlocks * MIXED_GRID_NT;
    long long one = 0, grid = 0;
    for (size_t k = 0; k + 1 < colOff.size(); k++) {
        int G = colOff[k + 1] - colOff[k];
        one += 2 * ((G + tOne - 1) / tOne);
        grid += 2 * ((G + tGrid - 1) / tGrid) + (gridBlocks > 1 ? 1 : 0);
    }
    if (one > grid) return 0;
    return mixed_smem(2, nc, nbodies, ng, ncol) <= (size_t)MIXED_SMEM_MAX ? 2 : 1;
}

void launch_pgs_mixed(const DBodies& B, DContacts& C, DPairs& P, const int* groupOrder, const int* colourOff,
                      int ncol, int nc, int iters, double omega, double comp, double tol, bool early, int fo,
                      double fv, double slide, double* Mj, double* K, float* F, float* BM, float* U, int4* GI,
                      int ng, int nbodies, int mcap, DCount* dc, int gridBlocks, int mode, cudaStream_t s,
                      double resTol, int check, int refine) {
    if (ncol <= 0 || nc <= 0) return;
    k_mixed_prep<<<(nc + 127) / 128, 128, 0, s>>>(B, C, nc, comp, omega, fo, fv, Mj, K, F, mcap);
    const int nk = std::max(ng, nbodies);
    k_mixed_groups<<<(nk + 127) / 128, 128, 0, s>>>(B, C, P, groupOrder, ng, GI, nbodies, BM);
    AM_LAUNCHED(2);
    int earlyI = early ? 1 : 0;
    if (mode == 1 || mode == 2) {   // one block: its sweep maxima and residuals live in shared memory
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_pgs_mixed<1, MIXED_ONE_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 MIXED_SMEM_MAX);
            cudaFuncSetAttribute(k_pgs_mixed<2, MIXED_ONE_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 MIXED_SMEM_MAX);
            attr = true;
        }
        auto kern = mode == 2 ? k_pgs_mixed<2, MIXED_ONE_NT> : k_pgs_mixed<1, MIXED_ONE_NT>;
        kern<<<1, MIXED_ONE_NT, mixed_smem(mode, nc, nbodies, ng, ncol), s>>>(
            B, C, P, colourOff, GI, ncol, nc, nbodies, iters, tol, earlyI, slide, Mj, K, F, BM, U, mcap, refine, dc,
            comp, resTol, check);
        AM_LAUNCHED(1);
        return;
    }
    cudaMemsetAsync(&dc->maxchg, 0, sizeof(dc->maxchg), s);
    cudaMemsetAsync(&dc->bar_count, 0, sizeof(int), s);
    cudaMemsetAsync(&dc->reschk, 0, sizeof(unsigned long long) * 4, s);
    DBodies Bc = B;
    const double* Mjc = Mj;
    const double* Kc = K;
    const int4* GIc = GI;
    void* args[] = {&Bc, &C, &P, (void*)&colourOff, (void*)&GIc, &ncol, &nc, &nbodies, &iters, &tol,
                    &earlyI, &slide, (void*)&Mjc, (void*)&Kc, (void*)&F, (void*)&BM, (void*)&U, &mcap, &refine,
                    &dc, &comp, &resTol, &check};
    cudaLaunchCooperativeKernel((void*)k_pgs_mixed<0, MIXED_GRID_NT>, dim3(gridBlocks), dim3(MIXED_GRID_NT),
                                args, 0, s);
    AM_LAUNCHED(1);
}

}  // namespace am
