// gs_exact.cu -- bit-exact projected Gauss-Seidel in the reference's contact
// order, parallelised by level scheduling.
//
// A Gauss-Seidel pass in list order (PGS.java:100-181) touches each body's
// delta-v as a chain of updates in list order.  Give contact i the level
// 1 + max(level of the previous contact on each of its dynamic bodies); then
// contacts of one level share no dynamic body, every contact of a lower level
// that shares a body precedes it in the list, and executing level by level
// reproduces the sequential pass bit for bit.  (Pinned bodies have
// minv = 0 and jinv = 0, so their delta-v stays +0 under any order.)
//
// Each contact is handled by one warp: lanes 0..11 own the Jacobian entries
// (a.v, a.w, b.v, b.w) and the matching delta-v components, J . dv is formed
// by shuffles in exactly the reference's association order
//   ((p0 + p1) + p2 + (p3 + p4) + p5) + ((p6 + p7) + p8 + (p9 + p10) + p11),
// and the multiplier update is evaluated uniformly by every lane with the
// reference's expression.  Levels are separated by the bounded grid barrier.
// Compiled with --fmad=false.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"
#include "grid_sync.cuh"

namespace am {
using namespace amd;

// J . dv in the reference's order; result valid in every lane
__device__ __forceinline__ double jdv_exact(double p) {
    const unsigned F = 0xffffffffu;
    double p1 = __shfl_down_sync(F, p, 1);
    double p2 = __shfl_down_sync(F, p, 2);
    double t = (p + p1) + p2;                    // lanes 0,3,6,9: dot of one 3-vector
    double u = t + __shfl_down_sync(F, t, 3);    // lanes 0,6: Vector6d.dot of one body
    double s = u + __shfl_down_sync(F, u, 6);    // lane 0: ja.dot(dv1) + jb.dot(dv2)
    return __shfl_sync(F, s, 0);
}

__device__ __forceinline__ double mu_exact(const DBodies& B, const DContacts& C, int c, int fo, double fv) {
    if (fo) return fv;
    double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
    if (f1 < 0.2 || f2 < 0.2) return jmin(f1, f2);
    if (f1 > 1. || f2 > 1.) return jmax(f1, f2);
    return (f1 + f2) / 2.;
}

// PGS.updateDeltaVwithLambdai for lane k: (minv * lambda) * J.v + dv on the
// linear lanes, lambda * (jinv J.w) + dv on the angular lanes.  One
// branch-free form serves every lane, (s * lambda) * e + dv with s = minv and
// e = J.v, or s = 1 and e = jinv J.w: 1 * lambda is lambda exactly, so the
// angular lanes round as lambda * e + dv does.  GB300 issues each FP64 warp
// instruction once for all lanes, so one form costs 3 instructions where
// per-lane branches cost one set per branch.
__device__ __forceinline__ double dv_update(double dv, double lam, bool act, double s, double e) {
    return act ? (s * lam) * e + dv : dv;
}

__global__ void k_gs_levels(DBodies B, DContacts C, const int* order, const int* levelOff, int nLevels, int iters,
                            double omega, double comp, double tol, int early, int fo, double fv, double slide,
                            DCount* dc) {
    const int nblocks = gridDim.x;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (nblocks * blockDim.x) >> 5;
    const int cap = C.cap;
    unsigned target = 0;
    const bool act = lane < 12;
    const int q = lane / 3;                 // 0 a.v, 1 a.w, 2 b.v, 3 b.w
    const int side = lane / 6;
    const int comp6 = lane % 6;

    // confidentWarmStart (PGS.java:250-256), in list order via the levels
    for (int L = 0; L < nLevels; L++) {
        for (int k = levelOff[L] + warp; k < levelOff[L + 1]; k += nwarps) {
            int c = order[k];
            int s1 = C.sb1[c], s2 = C.sb2[c];
            int body = side == 0 ? s1 : s2;
            double sc = (q == 0) ? B.minv[s1] : (q == 2) ? B.minv[s2] : 1.0;
            double dv = act ? __ldcg(B.dv + 6 * body + comp6) : 0.0;
            for (int r = 0; r < 3; r++) {
                double lam = C.lam[r * cap + c];
                double e = 0.0;
                if (q == 0 || q == 2) e = C.J[(12 * r + lane) * cap + c];
                else if (q == 1) e = C.Ia[(3 * r + comp6 - 3) * cap + c];
                else if (q == 3) e = C.Ib[(3 * r + comp6 - 3) * cap + c];
                dv = dv_update(dv, lam, act, sc, e);
            }
            if (act) __stcg(B.dv + 6 * body + comp6, dv);
        }
        if (!grid_barrier_counted(dc, nblocks, target)) return;
    }
    int iter = iters, done = 0;
    double change = 0;
    while (iter > 0) {
        const int par = done % 3;
        if (blockIdx.x == 0 && threadIdx.x == 0) dc->maxchg[(done + 1) % 3] = 0ull;   // the next sweep's slot
        double mx = 0;
        for (int L = 0; L < nLevels; L++) {
            for (int k = levelOff[L] + warp; k < levelOff[L + 1]; k += nwarps) {
                int c = order[k];
                int s1 = C.sb1[c], s2 = C.sb2[c];
                int body = side == 0 ? s1 : s2;
                double sc = (q == 0) ? B.minv[s1] : (q == 2) ? B.minv[s2] : 1.0;
                double dv = act ? __ldcg(B.dv + 6 * body + comp6) : 0.0;
                double j[3], e[3];
                for (int r = 0; r < 3; r++) {
                    j[r] = act ? C.J[(12 * r + lane) * cap + c] : 0.0;
                    e[r] = j[r];
                    if (q == 1) e[r] = C.Ia[(3 * r + comp6 - 3) * cap + c];
                    else if (q == 3) e[r] = C.Ib[(3 * r + comp6 - 3) * cap + c];
                }
                // normal direction
                double Jd = jdv_exact(j[0] * dv);
                double l0 = C.lam[c];
                double prev = l0;
                double D = C.bD[3 * cap + c];
                l0 = (D * l0 - omega * (C.bD[c] + Jd)) / (D + comp);
                l0 = jmax_i(0.0, l0);
                double diff = l0 - prev;
                dv = dv_update(dv, diff, act, sc, e[0]);
                mx = jmax_i(mx, abs_i(diff));
                double mu = mu_exact(B, C, c, fo, fv);
                double lr[3];
                lr[0] = l0;
                for (int r = 1; r < 3; r++) {
                    Jd = jdv_exact(j[r] * dv);
                    double l = C.lam[r * cap + c];
                    prev = l;
                    double Dr = C.bD[(3 + r) * cap + c];
                    l = (Dr * l - omega * (C.bD[r * cap + c] + Jd)) / (Dr + comp);
                    double lim = mu * l0;
                    l = jmax_i(l, neg_i(lim));
                    l = jmin_i(l, lim);
                    diff = l - prev;
                    dv = dv_update(dv, diff, act, sc, e[r]);
                    mx = jmax_i(mx, abs_i(diff));
                    lr[r] = l;
                }
                if (iter == 1) {   // Contact.updateContactState (Contact.java:385-398)
                    double w1 = C.bD[cap + c] + jdv_exact(j[1] * dv);
                    double w2 = C.bD[2 * cap + c] + jdv_exact(j[2] * dv);
                    int st;
                    if (fabs(l0) <= 1e-14) st = AM_STATE_BROKEN;
                    else if (fabs(w1) > slide) st = AM_STATE_ONEDGE;
                    else if (fabs(w2) > slide) st = AM_STATE_ONEDGE;
                    else st = AM_STATE_CLEAR;
                    if (lane == 0) C.state[c] = st;
                }
                if (lane == 0)
                    for (int r = 0; r < 3; r++) C.lam[r * cap + c] = lr[r];
                if (act) __stcg(B.dv + 6 * body + comp6, dv);
            }
            if (L == nLevels - 1 && lane == 0 && mx > 0)
                atomicMax(&dc->maxchg[par], (unsigned long long)__double_as_longlong(mx));
            if (!grid_barrier_counted(dc, nblocks, target)) return;
        }
        iter--;
        done++;
        change = __longlong_as_double((long long)*(volatile unsigned long long*)&dc->maxchg[par]);
        if (early && change < tol) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        dc->sweeps = done;
        dc->maxchg[0] = __double_as_longlong(change);
    }
}

// host: levels of a contact list (contact i's bodies s1[i], s2[i]; pinned
// bodies carry no dependency); returns contacts sorted by level
int gs_levels(const std::vector<int>& s1, const std::vector<int>& s2, const std::vector<int>& flags,
              std::vector<int>& order, std::vector<int>& levelOff, std::vector<int>& last) {
    int n = (int)s1.size();
    std::vector<int> lev(n);
    std::fill(last.begin(), last.end(), 0);
    int maxL = 0;
    for (int i = 0; i < n; i++) {
        int a = s1[i], b = s2[i];
        bool pa = flags[a] & F_PINNED, pb = flags[b] & F_PINNED;
        int l = 0;
        if (!pa) l = std::max(l, last[a]);
        if (!pb) l = std::max(l, last[b]);
        l++;
        if (!pa) last[a] = l;
        if (!pb) last[b] = l;
        lev[i] = l - 1;
        maxL = std::max(maxL, l);
    }
    levelOff.assign(maxL + 1, 0);
    for (int i = 0; i < n; i++) levelOff[lev[i] + 1]++;
    for (int L = 0; L < maxL; L++) levelOff[L + 1] += levelOff[L];
    std::vector<int> fill(levelOff.begin(), levelOff.end() - 1);
    order.assign(n, 0);
    for (int i = 0; i < n; i++) order[fill[lev[i]]++] = i;
    return maxL;
}

const void* gs_levels_kernel() { return (const void*)k_gs_levels; }

void launch_gs_levels(const DBodies& B, DContacts& C, const int* order, const int* levelOff, int nLevels, int iters,
                      double omega, double comp, double tol, bool early, int fo, double fv, double slide,
                      DCount* dc, int blocks, cudaStream_t s) {
    if (nLevels <= 0) return;
    cudaMemsetAsync(&dc->maxchg, 0, sizeof(dc->maxchg), s);
    cudaMemsetAsync(&dc->bar_count, 0, sizeof(int), s);
    int earlyI = early ? 1 : 0;
    DBodies Bc = B;
    void* args[] = {&Bc, &C, (void*)&order, (void*)&levelOff, &nLevels, &iters, &omega, &comp, &tol, &earlyI,
                    &fo, &fv, &slide, &dc};
    cudaLaunchCooperativeKernel((void*)k_gs_levels, dim3(blocks), dim3(128), args, 0, s);
    AM_LAUNCHED(1);
}

// Two blocks wait at a barrier whose target counts three: no arrival can
// complete it, so each block's wait must expire (or see the other's expiry).
__global__ void k_barrier_timeout_check(DCount* dc) {
    unsigned target = 0;
    grid_barrier_counted(dc, gridDim.x + 1, target);   // every block expects one arrival too many
}

void launch_barrier_timeout_check(DCount* dc, int spin_log2, cudaStream_t s) {
    cudaMemsetAsync(&dc->bar_count, 0, sizeof(int), s);
    cudaMemsetAsync(&dc->error, 0, sizeof(int), s);
    cudaMemcpyAsync(&dc->spin_log2, &spin_log2, sizeof(int), cudaMemcpyHostToDevice, s);
    k_barrier_timeout_check<<<2, 64, 0, s>>>(dc);
    AM_LAUNCHED(1);
    const int zero = 0;
    cudaMemcpyAsync(&dc->spin_log2, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
}

}  // namespace am
