// solve.cu -- warm start, solver setup and projected Gauss-Seidel on the device.
//
//  * warm start (CollisionProcessor.warmStart, CollisionProcessor.java:481-665):
//    the previous step's contacts are inserted in a hash table keyed like
//    Contact.hashCode/equals (unordered (body, bv) pair + info); duplicate keys
//    keep the later contact, as HashMap.put does.  One thread per body pair
//    walks that pair's contacts in list order: donors are only ever shared
//    inside one body pair (the key contains the pair), so the reference's
//    "take the multipliers and zero the donor" sequence is reproduced exactly.
//  * setup (Contact.computeB / computeJMinvJt, Contact.java:279-354) per
//    contact, plus jinv * J.w for each row and body (the angular part of
//    M^-1 J^T used by every delta-v update; same arithmetic as recomputing it).
//  * PGS (PGS.solve, PGS.java:73-256) in two orders:
//      - AM_ORDER_REFERENCE: list order, bit-identical to the reference
//        (level-scheduled kernel in gs_exact.cu);
//      - AM_ORDER_COLOURED: body-pair groups are greedily coloured so that no
//        two groups of one colour share a dynamic body (colouring here; the
//        sweep kernel is in pgs_fast.cu).
//
// Compiled with --fmad=false (see am_dev.cuh).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

// ---------------------------------------------------------------------------
// warm-start hash
__device__ __forceinline__ void ckey(const DContacts& C, int c, int info, int k[5]) {
    int a = C.b1[c], b = C.b2[c], va = C.bv1[c], vb = C.bv2[c];
    if (a < b || (a == b && va <= vb)) { k[0] = a; k[1] = va; k[2] = b; k[3] = vb; }
    else { k[0] = b; k[1] = vb; k[2] = a; k[3] = va; }
    k[4] = info;
}
__device__ __forceinline__ unsigned khash(const int k[5]) {
    unsigned h = 2166136261u;
    for (int i = 0; i < 5; i++) { h ^= (unsigned)k[i]; h *= 16777619u; h ^= h >> 15; }
    return h;
}
__device__ __forceinline__ bool keq(const int a[5], const int b[5]) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3] && a[4] == b[4];
}

__global__ void k_ws_build(DContacts P, int nprev, DHash H) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nprev) return;
    int k[5];
    ckey(P, i, P.info[i], k);
    unsigned m = (unsigned)H.cap - 1u;
    unsigned h = khash(k) & m;
    for (int probe = 0; probe < H.cap; probe++, h = (h + 1) & m) {
        int old = atomicCAS(&H.slot[h], -1, i);
        if (old == -1) return;
        int k2[5];
        ckey(P, old, P.info[old], k2);
        if (keq(k, k2)) { atomicMax(&H.slot[h], i); return; }
    }
}

void launch_ws_build(const DContacts& prev, int nprev, DHash& H, cudaStream_t s) {
    cudaMemsetAsync(H.slot, 0xff, sizeof(int) * H.cap, s);
    if (nprev > 0) { k_ws_build<<<(nprev + 255) / 256, 256, 0, s>>>(prev, nprev, H); AM_LAUNCHED(1); }
}

__device__ int ws_lookup(const DContacts& cur, int c, int info, const DContacts& P, const DHash& H) {
    int k[5];
    ckey(cur, c, info, k);
    unsigned m = (unsigned)H.cap - 1u;
    unsigned h = khash(k) & m;
    for (int probe = 0; probe < H.cap; probe++, h = (h + 1) & m) {
        int s = H.slot[h];
        if (s < 0) return -1;
        int k2[5];
        ckey(P, s, P.info[s], k2);
        if (keq(k, k2)) return s;
    }
    return -1;
}

__device__ __forceinline__ v3 cworld(const DBodies& B, const DContacts& C, int c) {
    int b = C.b1[c];
    int cap = C.cap;
    v3 p = mk(C.f[0 * cap + c], C.f[1 * cap + c], C.f[2 * cap + c]);
    return tpoint(ldm(B.R + 9 * b), ldv(B.x + 3 * b), p);
}

__device__ void take_old(DContacts& C, int c, DContacts& P, int o, bool zeroDonor) {
    int cap = C.cap, pc = P.cap;
    C.fresh[c] = 0;
    for (int r = 0; r < 3; r++) {
        double l = P.lam[r * pc + o];
        C.lam[r * cap + c] = l;
        C.lamw[r * cap + c] = l;
    }
    if (zeroDonor)
        for (int r = 0; r < 3; r++) P.lam[r * pc + o] = 0.0;
    C.pcv[c] = P.cv[o];
}

__global__ void k_warm_start(DBodies B, DContacts C, DContacts P, DHash H, DPairs PR, int npairs, int nprev) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int n = PR.count[p], off = PR.off[p];
    if (n == 0) return;
    int a = PR.a[p], b = PR.b[p];
    bool bothBox = B.type[a] == AM_BOX && B.type[b] == AM_BOX;
    for (int c = off; c < off + n; c++) {
        if (nprev == 0) { C.fresh[c] = 1; continue; }
        if (!bothBox) {   // vanillaWarmStart
            int o = ws_lookup(C, c, C.info[c], P, H);
            if (o >= 0) take_old(C, c, P, o, false);
            else C.fresh[c] = 1;
            continue;
        }
        v3 pNew = cworld(B, C, c);
        int myInfo = C.info[c];
        int o = ws_lookup(C, c, myInfo, P, H);
        if (o >= 0) {
            double d = dist(pNew, cworld(B, P, o));
            if (d > 0.05) {
                double best = d;
                int bestO = o;
                for (int info = 0; info < 9; info++) {
                    if (info == myInfo) continue;
                    int o2 = ws_lookup(C, c, info, P, H);
                    if (o2 < 0) break;
                    double d2 = dist(pNew, cworld(B, P, o2));
                    if (d2 < best) { best = d2; bestO = o2; }
                }
                o = bestO;
                d = best;
            }
            if (d < 0.05) take_old(C, c, P, o, true);
            else C.fresh[c] = 1;
        } else {
            double best = 1.79769313486231570e308;
            int bestO = -1;
            for (int info = 0; info < 9; info++) {
                int o2 = ws_lookup(C, c, info, P, H);
                if (o2 < 0) break;
                double d2 = dist(pNew, cworld(B, P, o2));
                if (d2 < best) { best = d2; bestO = o2; }
            }
            if (bestO >= 0) {
                if (best < 0.05) take_old(C, c, P, bestO, true);
            } else {
                C.fresh[c] = 1;
            }
        }
    }
}

void launch_warm_start(const DBodies& B, DContacts& cur, DContacts& prev, const DHash& H, DPairs& P,
                       int npairs, int nprev, cudaStream_t s) {
    if (npairs <= 0) return;
    k_warm_start<<<(npairs + 127) / 128, 128, 0, s>>>(B, cur, prev, H, P, npairs, nprev);
    AM_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
// setup: Contact.computeB + computeJMinvJt, angular M^-1 J^T parts
__device__ __forceinline__ v3 Jrow(const DContacts& C, int c, int q) {
    int cap = C.cap;
    return mk(C.J[(3 * q) * cap + c], C.J[(3 * q + 1) * cap + c], C.J[(3 * q + 2) * cap + c]);
}

__global__ void k_solve_prep(DBodies B, DContacts C, int nc, double dt, double fb, int inColl, int restOv,
                             double restVal, int redoWarm) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int cap = C.cap;
    int r1 = C.b1[c], r2 = C.b2[c];
    int s1 = inColl ? r1 : C.sb1[c];
    int s2 = inColl ? r2 : C.sb2[c];
    if (redoWarm)
        for (int r = 0; r < 3; r++) C.lam[r * cap + c] = C.lamw[r * cap + c];
    double restitution = (B.restitution[r1] + B.restitution[r2]) / 2.;
    if (restOv) restitution = restVal;
    v3 J[12];
    for (int q = 0; q < 12; q++) J[q] = Jrow(C, c, q);
    double bn = 0, bt1 = 0, bt2 = 0;
    for (int side = 0; side < 2; side++) {
        int sb = side == 0 ? s1 : s2;
        int o = side == 0 ? 0 : 2;   // row offsets: a rows 0,4,8 / b rows 2,6,10
        v3 v = ldv(B.v + 3 * sb), w = ldv(B.w + 3 * sb);
        m3 jinv = ldm(B.jinv + 9 * sb);
        v3 t = scaleadd(B.minv[sb] * dt, ldv(B.force + 3 * sb), v);
        bn += dot(t, J[o]); bt1 += dot(t, J[4 + o]); bt2 += dot(t, J[8 + o]);
        t = mxv(jinv, ldv(B.torque + 3 * sb));
        t.x *= dt; t.y *= dt; t.z *= dt;
        t = add(t, w);
        bn += dot(t, J[o + 1]); bt1 += dot(t, J[4 + o + 1]); bt2 += dot(t, J[8 + o + 1]);
        double bb = dot(v, J[o]) + dot(w, J[o + 1]);
        bb *= restitution;
        bn += bb;
    }
    bn += fb * C.cv[c];
    C.bD[0 * cap + c] = bn; C.bD[1 * cap + c] = bt1; C.bD[2 * cap + c] = bt2;
    m3 ja = ldm(B.jinv + 9 * s1), jb = ldm(B.jinv + 9 * s2);
    double m1 = B.minv[s1], m2 = B.minv[s2];
    for (int r = 0; r < 3; r++) {
        v3 ta = mxv(ja, J[4 * r + 1]);
        v3 tb = mxv(jb, J[4 * r + 3]);
        double D = m1 * dot(J[4 * r], J[4 * r]) + dot(J[4 * r + 1], ta) + m2 * dot(J[4 * r + 2], J[4 * r + 2]) + dot(J[4 * r + 3], tb);
        C.bD[(3 + r) * cap + c] = D;
        C.Ia[(3 * r) * cap + c] = ta.x; C.Ia[(3 * r + 1) * cap + c] = ta.y; C.Ia[(3 * r + 2) * cap + c] = ta.z;
        C.Ib[(3 * r) * cap + c] = tb.x; C.Ib[(3 * r + 1) * cap + c] = tb.y; C.Ib[(3 * r + 2) * cap + c] = tb.z;
    }
    if (inColl) { C.sb1[c] = s1; C.sb2[c] = s2; }
}

void launch_solve_prep(const DBodies& B, DContacts& C, int nc, double dt, double fb, bool inColl, int restOv,
                       double restVal, int redoWarm, cudaStream_t s) {
    if (nc <= 0) return;
    k_solve_prep<<<(nc + 127) / 128, 128, 0, s>>>(B, C, nc, dt, fb, inColl ? 1 : 0, restOv, restVal, redoWarm);
    AM_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
// one contact row update: Jdv, projected multiplier, delta-v update
struct RowCtx {
    double omega, comp;
};

__device__ __forceinline__ double mu_of(const DBodies& B, const DContacts& C, int c, int fo, double fv) {
    if (fo) return fv;
    double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
    if (f1 < 0.2 || f2 < 0.2) return jmin(f1, f2);
    if (f1 > 1. || f2 > 1.) return jmax(f1, f2);
    return (f1 + f2) / 2.;
}

// dv loads/stores go through L2 (.cg) so that blocks on other SMs see them
// after a grid barrier.
__device__ __forceinline__ v3 ldcg3(const double* p) { return mk(__ldcg(p), __ldcg(p + 1), __ldcg(p + 2)); }
__device__ __forceinline__ void stcg3(double* p, v3 a) { __stcg(p, a.x); __stcg(p + 1, a.y); __stcg(p + 2, a.z); }

// PGS.updateDeltaVwithLambdai (PGS.java:221-245) with jinv*J.w precomputed
__device__ __forceinline__ void apply_dv(const DBodies& B, const DContacts& C, int c, int r, double lambda,
                                         int s1, int s2, v3 Jav, v3 Jbv) {
    int cap = C.cap;
    v3 ia = mk(C.Ia[(3 * r) * cap + c], C.Ia[(3 * r + 1) * cap + c], C.Ia[(3 * r + 2) * cap + c]);
    v3 ib = mk(C.Ib[(3 * r) * cap + c], C.Ib[(3 * r + 1) * cap + c], C.Ib[(3 * r + 2) * cap + c]);
    double* d1 = B.dv + 6 * s1;
    double* d2 = B.dv + 6 * s2;
    stcg3(d1, scaleadd(B.minv[s1] * lambda, Jav, ldcg3(d1)));
    stcg3(d1 + 3, scaleadd(lambda, ia, ldcg3(d1 + 3)));
    stcg3(d2, scaleadd(B.minv[s2] * lambda, Jbv, ldcg3(d2)));
    stcg3(d2 + 3, scaleadd(lambda, ib, ldcg3(d2 + 3)));
}

__device__ __forceinline__ double jdv(const DBodies& B, int s1, int s2, v3 Jav, v3 Jaw, v3 Jbv, v3 Jbw) {
    const double* d1 = B.dv + 6 * s1;
    const double* d2 = B.dv + 6 * s2;
    return (dot(Jav, ldcg3(d1)) + dot(Jaw, ldcg3(d1 + 3))) + (dot(Jbv, ldcg3(d2)) + dot(Jbw, ldcg3(d2 + 3)));
}

// the three rows of one contact in one sweep; returns max |delta lambda|
__device__ double contact_sweep(const DBodies& B, DContacts& C, int c, double omega, double comp, int fo,
                                double fv, bool last, double slide) {
    int cap = C.cap;
    int s1 = C.sb1[c], s2 = C.sb2[c];
    double mx = 0;
    double l0 = C.lam[c];
    // normal row
    {
        v3 av = Jrow(C, c, 0), aw = Jrow(C, c, 1), bv = Jrow(C, c, 2), bw = Jrow(C, c, 3);
        double Jd = jdv(B, s1, s2, av, aw, bv, bw);
        double D = C.bD[3 * cap + c];
        double prev = l0;
        l0 = (D * l0 - omega * (C.bD[c] + Jd)) / (D + comp);
        l0 = jmax(0.0, l0);
        double diff = l0 - prev;
        apply_dv(B, C, c, 0, diff, s1, s2, av, bv);
        mx = jmax(mx, fabs(diff));
        C.lam[c] = l0;
    }
    double mu = mu_of(B, C, c, fo, fv);
    double w1 = 0, w2 = 0;
    for (int r = 1; r < 3; r++) {
        v3 av = Jrow(C, c, 4 * r), aw = Jrow(C, c, 4 * r + 1), bv = Jrow(C, c, 4 * r + 2), bw = Jrow(C, c, 4 * r + 3);
        double Jd = jdv(B, s1, s2, av, aw, bv, bw);
        double D = C.bD[(3 + r) * cap + c];
        double l = C.lam[r * cap + c];
        double prev = l;
        l = (D * l - omega * (C.bD[r * cap + c] + Jd)) / (D + comp);
        double lim = mu * l0;
        l = jmax(l, -lim);
        l = jmin(l, lim);
        double diff = l - prev;
        apply_dv(B, C, c, r, diff, s1, s2, av, bv);
        mx = jmax(mx, fabs(diff));
        C.lam[r * cap + c] = l;
    }
    if (last) {   // Contact.updateContactState (Contact.java:385-398)
        for (int r = 1; r < 3; r++) {
            v3 av = Jrow(C, c, 4 * r), aw = Jrow(C, c, 4 * r + 1), bv = Jrow(C, c, 4 * r + 2), bw = Jrow(C, c, 4 * r + 3);
            double w = C.bD[r * cap + c] + jdv(B, s1, s2, av, aw, bv, bw);
            if (r == 1) w1 = w; else w2 = w;
        }
        int st;
        if (fabs(l0) <= 1e-14) st = AM_STATE_BROKEN;
        else if (fabs(w1) > slide) st = AM_STATE_ONEDGE;
        else if (fabs(w2) > slide) st = AM_STATE_ONEDGE;
        else st = AM_STATE_CLEAR;
        C.state[c] = st;
    }
    return mx;
}

__device__ void warm_apply(const DBodies& B, const DContacts& C, int c) {
    int cap = C.cap;
    int s1 = C.sb1[c], s2 = C.sb2[c];
    for (int r = 0; r < 3; r++)
        apply_dv(B, C, c, r, C.lam[r * cap + c], s1, s2, Jrow(C, c, 4 * r), Jrow(C, c, 4 * r + 2));
}

// ---------------------------------------------------------------------------
// colouring of body-pair groups: Jones-Plassmann rounds with first-fit
// colours.  Each round, every uncoloured group whose priority is the largest
// among the uncoloured groups at each of its dynamic bodies takes the
// smallest colour not yet used at either body.  Groups selected in one round
// share no dynamic body, so the per-body colour masks (maxC bits) need no
// atomics between them; groups of one colour never share a dynamic body, so
// they can update delta-v concurrently.  A chain of groups (a stack) takes
// three colours at most.  Groups with more contacts go first (low colours),
// ties broken by a hash, made unique by the group index.
__device__ __forceinline__ unsigned long long prio(const DPairs& P, int g) {
    unsigned h = (unsigned)g * 2654435761u;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15;
    unsigned long long cnt = (unsigned long long)min(P.count[g], 255);
    return (cnt << 56) | ((unsigned long long)(h & 0xFFFFFFu) << 32) | (unsigned)g;
}

__global__ void k_colour(DBodies B, DContacts C, DPairs P, int npairs, int* colourOf, int* colourCnt, int maxC,
                         unsigned long long* bodyMax, unsigned long long* used, int nbodies, DCount* dc) {
    __shared__ int s_left, s_full, s_ncol;
    const int W = (maxC + 63) / 64;   // 64-bit words of a body's colour mask
    int t = threadIdx.x, T = blockDim.x;
    for (int g = t; g < npairs; g += T) colourOf[g] = (P.count[g] > 0) ? -1 : -2;
    for (int b = t; b < nbodies * W; b += T) used[b] = 0ull;
    if (t == 0) { s_full = 0; s_ncol = 0; s_left = 1; }
    __syncthreads();
    const int maxRounds = 1 << 16;
    for (int round = 0; round < maxRounds; round++) {
        for (int b = t; b < nbodies; b += T) bodyMax[b] = 0ull;
        __syncthreads();
        if (t == 0) s_left = 0;
        for (int g = t; g < npairs; g += T) {
            if (colourOf[g] != -1) continue;
            int c = P.off[g];
            int s1 = C.sb1[c], s2 = C.sb2[c];
            unsigned long long pr = prio(P, g);
            if (!(B.flags[s1] & F_PINNED)) atomicMax(&bodyMax[s1], pr);
            if (!(B.flags[s2] & F_PINNED)) atomicMax(&bodyMax[s2], pr);
        }
        __syncthreads();
        for (int g = t; g < npairs; g += T) {
            if (colourOf[g] != -1) continue;
            int c = P.off[g];
            int s1 = C.sb1[c], s2 = C.sb2[c];
            bool p1 = B.flags[s1] & F_PINNED, p2 = B.flags[s2] & F_PINNED;
            unsigned long long pr = prio(P, g);
            if (!((p1 || bodyMax[s1] == pr) && (p2 || bodyMax[s2] == pr))) { atomicAdd(&s_left, 1); continue; }
            int col = -1;
            for (int w = 0; w < W && col < 0; w++) {
                unsigned long long m = (p1 ? 0ull : used[(size_t)s1 * W + w]) | (p2 ? 0ull : used[(size_t)s2 * W + w]);
                if (m != ~0ull) col = 64 * w + __ffsll((long long)~m) - 1;
            }
            if (col < 0 || col >= maxC) { colourOf[g] = -2; s_full = 1; continue; }   // more than maxC colours
            if (!p1) used[(size_t)s1 * W + col / 64] |= 1ull << (col % 64);
            if (!p2) used[(size_t)s2 * W + col / 64] |= 1ull << (col % 64);
            colourOf[g] = col;
            atomicAdd(&colourCnt[col], 1);
            atomicMax(&s_ncol, col + 1);
        }
        __syncthreads();
        int left = s_left;
        __syncthreads();
        if (left == 0) break;
    }
    if (t == 0) {
        dc->n_colours = s_ncol;
        if (s_left != 0 || s_full) dc->error = AM_E_CAPACITY;
    }
}

// Small scenes: sequential first-fit in group order (the broad phase's
// (i, j) order), one thread over shared-memory copies of the groups' bodies
// and the bodies' colour masks.  A stack of bodies, whose groups come in
// order along the stack, takes two colours (Jones-Plassmann up to three),
// and a colour costs the single-scene sweep a barrier and a group chain.
__global__ void k_colour_seq(DBodies B, DContacts C, DPairs P, int npairs, int* colourOf, int* colourCnt, int maxC,
                             int nbodies, DCount* dc) {
    extern __shared__ unsigned long long sq[];
    const int W = (maxC + 63) / 64;
    unsigned long long* used = sq;                                    // nbodies * W
    int2* gb = reinterpret_cast<int2*>(sq + (size_t)nbodies * W);     // npairs
    int* cnt = reinterpret_cast<int*>(gb + npairs);                   // maxC
    const int t = threadIdx.x, T = blockDim.x;
    const int PIN = (int)0x80000000u;
    for (int b = t; b < nbodies * W; b += T) used[b] = 0ull;
    for (int k = t; k < maxC; k += T) cnt[k] = 0;
    for (int g = t; g < npairs; g += T) {
        if (P.count[g] <= 0) { gb[g] = make_int2(-1, -1); continue; }
        const int c = P.off[g];
        const int s1 = C.sb1[c], s2 = C.sb2[c];
        gb[g] = make_int2(s1 | ((B.flags[s1] & F_PINNED) ? PIN : 0), s2 | ((B.flags[s2] & F_PINNED) ? PIN : 0));
    }
    __syncthreads();
    __shared__ int s_ncol, s_full;
    if (t == 0) {
        int ncol = 0, full = 0;
        for (int g = 0; g < npairs; g++) {
            const int2 q = gb[g];
            if (q.x == -1 && q.y == -1) { colourOf[g] = -2; continue; }
            const bool p1 = q.x < 0, p2 = q.y < 0;
            const int s1 = q.x & 0x7fffffff, s2 = q.y & 0x7fffffff;
            int col = -1;
            for (int w = 0; w < W && col < 0; w++) {
                unsigned long long m = (p1 ? 0ull : used[(size_t)s1 * W + w]) | (p2 ? 0ull : used[(size_t)s2 * W + w]);
                if (m != ~0ull) col = 64 * w + __ffsll((long long)~m) - 1;
            }
            if (col < 0 || col >= maxC) { colourOf[g] = -2; full = 1; continue; }
            if (!p1) used[(size_t)s1 * W + col / 64] |= 1ull << (col % 64);
            if (!p2) used[(size_t)s2 * W + col / 64] |= 1ull << (col % 64);
            colourOf[g] = col;
            cnt[col]++;
            ncol = max(ncol, col + 1);
        }
        s_ncol = ncol;
        s_full = full;
    }
    __syncthreads();
    for (int k = t; k < maxC; k += T) colourCnt[k] = cnt[k];
    if (t == 0) {
        dc->n_colours = s_ncol;
        if (s_full) dc->error = AM_E_CAPACITY;
    }
}

__global__ void k_colour_place(DPairs P, int npairs, const int* colourOf, const int* colourOff, int* fill,
                               int* groupOrder) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= npairs) return;
    int c = colourOf[g];
    if (c < 0) return;
    int pos = colourOff[c] + atomicAdd(&fill[c], 1);
    groupOrder[pos] = g;
}

// host-side launcher of the colouring (needs the contact buffer for solve bodies)
void colour_groups(const DBodies& B, const DContacts& C, DPairs& P, int npairs, int* colourOf, int* colourCnt,
                   int* colourOff, int* fill, int* groupOrder, int maxC, unsigned long long* bodyMax, int nbodies,
                   DCount* dc, Scratch& sc, cudaStream_t s) {
    if (npairs <= 0) { cudaMemsetAsync(&dc->n_colours, 0, sizeof(int), s); return; }
    cudaMemsetAsync(colourCnt, 0, sizeof(int) * (maxC + 1), s);
    const int W = (maxC + 63) / 64;
    const size_t seqSmem = 8 * (size_t)nbodies * W + 8 * (size_t)npairs + 4 * (size_t)maxC;
    if (npairs <= 128 && seqSmem <= 48 * 1024)
        k_colour_seq<<<1, 256, seqSmem, s>>>(B, C, P, npairs, colourOf, colourCnt, maxC, nbodies, dc);
    else
        k_colour<<<1, 1024, 0, s>>>(B, C, P, npairs, colourOf, colourCnt, maxC, bodyMax, bodyMax + nbodies,
                                    nbodies, dc);
    AM_LAUNCHED(1);
    launch_scan(colourCnt, colourOff, maxC + 1, sc, nullptr, s);
    cudaMemsetAsync(fill, 0, sizeof(int) * maxC, s);
    k_colour_place<<<(npairs + 255) / 256, 256, 0, s>>>(P, npairs, colourOf, colourOff, fill, groupOrder);
    AM_LAUNCHED(1);
}

__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = jmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---------------------------------------------------------------------------
// natural-map LCP residual at the final state: w = b + J dv + c lambda,
// r = lambda - proj(lambda - w / (D + c)) per row; inf-norms via atomicMax
__global__ void k_residual(DBodies B, DContacts C, int nc, double comp, int fo, double fv, DCount* dc) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    double rmax = 0, lmax = 0;
    if (c < nc) {
        int cap = C.cap;
        int s1 = C.sb1[c], s2 = C.sb2[c];
        double lam[3], w[3];
        for (int r = 0; r < 3; r++) {
            lam[r] = C.lam[r * cap + c];
            double Jd = jdv(B, s1, s2, Jrow(C, c, 4 * r), Jrow(C, c, 4 * r + 1), Jrow(C, c, 4 * r + 2), Jrow(C, c, 4 * r + 3));
            w[r] = C.bD[r * cap + c] + Jd + comp * lam[r];
        }
        double mu = mu_of(B, C, c, fo, fv);
        double z0 = lam[0] - w[0] / (C.bD[3 * cap + c] + comp);
        double r0 = lam[0] - (z0 > 0 ? z0 : 0.0);
        rmax = fabs(r0);
        lmax = fabs(lam[0]);
        for (int r = 1; r < 3; r++) {
            double z = lam[r] - w[r] / (C.bD[(3 + r) * cap + c] + comp);
            double lim = mu * lam[0];
            z = z < -lim ? -lim : (z > lim ? lim : z);
            rmax = fmax(rmax, fabs(lam[r] - z));
            lmax = fmax(lmax, fabs(lam[r]));
        }
    }
    rmax = warp_max(rmax);
    lmax = warp_max(lmax);
    if ((threadIdx.x & 31) == 0) {
        atomicMax((unsigned long long*)&dc->res_abs, (unsigned long long)__double_as_longlong(rmax));
        atomicMax((unsigned long long*)&dc->lam_max, (unsigned long long)__double_as_longlong(lmax));
    }
}

void launch_residual(const DBodies& B, DContacts& C, int nc, double comp, int fo, double fv, DCount* dc,
                     cudaStream_t s) {
    cudaMemsetAsync(&dc->res_abs, 0, sizeof(double) * 2, s);
    if (nc <= 0) return;
    k_residual<<<(nc + 255) / 256, 256, 0, s>>>(B, C, nc, comp, fo, fv, dc);
    AM_LAUNCHED(1);
}

// CollisionProcessor.clearBodyPairContacts: a pair survives when one of its
// contacts has |lambda_n| > 1e-14 (CollisionProcessor.java:213-226)
__global__ void k_bpc_keep(DContacts C, DPairs P, int npairs) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int keep = 0;
    for (int c = P.off[p]; c < P.off[p] + P.count[p]; c++)
        if (fabs(C.lam[c]) > 1e-14) keep = 1;
    P.keep[p] = keep;
}

void launch_bpc_keep(const DContacts& C, DPairs& P, int npairs, cudaStream_t s) {
    if (npairs <= 0) return;
    k_bpc_keep<<<(npairs + 255) / 256, 256, 0, s>>>(C, P, npairs);
    AM_LAUNCHED(1);
}

}  // namespace am
