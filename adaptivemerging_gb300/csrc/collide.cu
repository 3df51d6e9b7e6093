// collide.cu -- collision detection on the device: world centres of the
// sphere-tree nodes, broad phase over the top-level body list, expansion of
// collection pairs into sub-body pairs, and the narrow phase (box-box,
// box-plane, box-sphere, sphere-tree traversals) with the contact setup
// (Contact.set: tangent frame, Jacobian rows, body-1 frame) fused into the
// emitting pass.
//
// Order contract: contacts are written in exactly the order the reference's
// CollisionProcessor.broadPhase / narrowPhase recursion creates them
// (CollisionProcessor.java:683-757): pairs (i<j) over the top-level list in
// row-major order, collection sub-bodies outer-then-inner, tree traversal in
// depth-first child order, collider emission order inside a pair.  The
// broad phase keeps a pair only when the reference's own first quick-exit
// test of that pair passes, evaluated with the same FP64 expression, so the
// candidate set is exact, not approximate.
//
// Compiled with --fmad=false: every predicate and every contact quantity is
// bit-identical to the reference arithmetic.
#include <cuda_runtime.h>

#include "am_ctx.hpp"
#include "am_dev.cuh"

namespace am {
using namespace amd;

long long g_launches = 0;

// ---------------------------------------------------------------------------
// exclusive scan of int32 (block-local scan, scan of block sums, add)
static const int SCAN_T = 256, SCAN_E = 4, SCAN_B = SCAN_T * SCAN_E;

__global__ void k_scan_block(const int* in, int* out, int n, int* blockSums) {
    __shared__ int s[SCAN_T];
    int base = blockIdx.x * SCAN_B + threadIdx.x * SCAN_E;
    int v[SCAN_E], sum = 0;
    for (int k = 0; k < SCAN_E; k++) { v[k] = (base + k < n) ? in[base + k] : 0; sum += v[k]; }
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < SCAN_T; off <<= 1) {
        int t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    int run = s[threadIdx.x] - sum;
    for (int k = 0; k < SCAN_E; k++) { if (base + k < n) out[base + k] = run; run += v[k]; }
    if (threadIdx.x == SCAN_T - 1) blockSums[blockIdx.x] = s[SCAN_T - 1];
}

__global__ void k_scan_sums(int* sums, int nb, int* total) {
    // single block; nb <= SCAN_B
    __shared__ int s[SCAN_T];
    int base = threadIdx.x * SCAN_E;
    int v[SCAN_E], sum = 0;
    for (int k = 0; k < SCAN_E; k++) { v[k] = (base + k < nb) ? sums[base + k] : 0; sum += v[k]; }
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < SCAN_T; off <<= 1) {
        int t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    int run = s[threadIdx.x] - sum;
    for (int k = 0; k < SCAN_E; k++) { if (base + k < nb) sums[base + k] = run; run += v[k]; }
    if (threadIdx.x == SCAN_T - 1 && total) *total = s[SCAN_T - 1];
}

__global__ void k_scan_add(int* out, int n, const int* sums) {
    int i = blockIdx.x * SCAN_B + threadIdx.x;
    int add = sums[blockIdx.x];
    for (int k = 0; k < SCAN_E; k++, i += SCAN_T)
        if (i < n) out[i] += add;
}

void launch_scan(const int* in, int* out, int n, Scratch& sc, int* total, cudaStream_t s) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(int), s);
        return;
    }
    int nb = (n + SCAN_B - 1) / SCAN_B;
    k_scan_block<<<nb, SCAN_T, 0, s>>>(in, out, n, sc.block);
    AM_LAUNCHED(1);
    if (nb <= SCAN_B) {
        k_scan_sums<<<1, SCAN_T, 0, s>>>(sc.block, nb, total);
        AM_LAUNCHED(1);
    } else {   // more than 2^20 entries: the block sums are scanned in the same way, in place
        const int nb2 = (nb + SCAN_B - 1) / SCAN_B;   // <= SCAN_B for n <= 2^30
        int* b2 = sc.block + sc.cap_block - SCAN_B;
        k_scan_block<<<nb2, SCAN_T, 0, s>>>(sc.block, sc.block, nb, b2);
        k_scan_sums<<<1, SCAN_T, 0, s>>>(b2, nb2, total);
        k_scan_add<<<nb2, SCAN_T, 0, s>>>(sc.block, nb, b2);
        AM_LAUNCHED(3);
    }
    if (nb > 1) { k_scan_add<<<nb, SCAN_T, 0, s>>>(out, n, sc.block); AM_LAUNCHED(1); }
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ m3 bodyR(const DBodies& B, int i) { return ldm(B.R + 9 * i); }
__device__ __forceinline__ v3 bodyX(const DBodies& B, int i) { return ldv(B.x + 3 * i); }

__global__ void k_bv_update(DBodies B, DNodes N) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N.n) return;
    int b = N.body[k];
    m3 R = bodyR(B, b);
    v3 c = tpoint(R, bodyX(B, b), ldv(N.cB + 3 * k));   // BVSphere.updatecW
    stv(N.cW + 3 * k, c);
}

void launch_bv_update(const DBodies& B, const DNodes& N, cudaStream_t s) {
    if (N.n == 0) return;
    k_bv_update<<<(N.n + 255) / 256, 256, 0, s>>>(B, N);
    AM_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
// Broad phase.  The reference test order is: skip pinned-pinned and
// pinned-sleeping pairs (CollisionProcessor.java:693-694), then the narrow
// phase, whose first statement for every primitive pair is a quick exit.
__device__ bool pair_may_touch(const DBodies& B, const DNodes& N, int a, int b) {
    int fa = B.flags[a], fb = B.flags[b];
    bool pa = fa & F_PINNED, pb = fb & F_PINNED;
    if (pa && pb) return false;
    if ((pa && (fb & F_SLEEPING)) || (pb && (fa & F_SLEEPING))) return false;
    if ((fa & F_COLLECTION) || (fb & F_COLLECTION)) return true;  // brute force over sub-bodies
    int ta = B.type[a], tb = B.type[b];
    if (ta == AM_PLANE && tb == AM_PLANE) return false;
    if (ta == AM_PLANE || tb == AM_PLANE) {
        int pl = ta == AM_PLANE ? a : b, o = ta == AM_PLANE ? b : a;
        v3 n = ldv(B.plane + 4 * pl);
        double d = B.plane[4 * pl + 3];
        if (B.type[o] == AM_BOX) {       // BoxPlane.java:29
            v3 x = bodyX(B, o);
            return !(x.x * n.x + x.y * n.y + x.z * n.z + d > B.radius[o]);
        }
        int r0 = B.root[o];              // collideSphereTreeAndPlane root test (CollisionProcessor.java:802)
        v3 c = ldv(N.cW + 3 * r0);
        double dd = n.x * c.x + n.y * c.y + n.z * c.z + d - N.r[r0];
        return dd < 0;
    }
    if (ta == AM_BOX && tb == AM_BOX) {  // BoxBox.java:466
        v3 p = sub(bodyX(B, b), bodyX(B, a));
        return !(length(p) > B.radius[a] + B.radius[b]);
    }
    if (ta == AM_BOX || tb == AM_BOX) {  // BoxSphere.dBoxSphereTest first exit (BoxSphere.java:157)
        int bx = ta == AM_BOX ? a : b, t = ta == AM_BOX ? b : a;
        int r0 = B.root[t];
        v3 c = ldv(N.cW + 3 * r0);
        return !(dist(c, bodyX(B, bx)) > B.radius[bx] + N.r[r0]);
    }
    int r1 = B.root[a], r2 = B.root[b];  // BVSphere.intersects (BVSphere.java:184-186)
    double rr = N.r[r1] + N.r[r2];
    return dist2(ldv(N.cW + 3 * r1), ldv(N.cW + 3 * r2)) < rr * rr;
}

// Bounding centre and radius of every top-level body in FP32 for a
// conservative prefilter: boxes use (x, radius) of BoxBox / BoxSphere's
// quick exit, sphere trees their root node (cW, r); planes and collections
// get w = -1 and always take the exact test.
__global__ void k_broad_pack(DBodies B, DNodes N, const int* top, int ntop) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int a = top[i];
    int t = B.type[a];
    float4 c = make_float4(0.f, 0.f, 0.f, -1.f);
    if (!(B.flags[a] & F_COLLECTION) && t != AM_PLANE) {
        if (t == AM_BOX) {
            v3 x = bodyX(B, a);
            c = make_float4((float)x.x, (float)x.y, (float)x.z, (float)B.radius[a]);
        } else {
            int r0 = B.root[a];
            v3 x = ldv(N.cW + 3 * r0);
            c = make_float4((float)x.x, (float)x.y, (float)x.z, (float)N.r[r0]);
        }
    }
    B.bc[a] = c;
}

// the same bounds for the bodies inside collections (their own box or tree;
// the expansion of a collection's candidates tests its members with them)
__global__ void k_broad_pack_subs(DBodies B, DNodes N, const int* subIds, int nsub) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsub) return;
    int a = subIds[i];
    int t = B.type[a];
    float4 c = make_float4(0.f, 0.f, 0.f, -1.f);
    if (t == AM_BOX) {
        v3 x = bodyX(B, a);
        c = make_float4((float)x.x, (float)x.y, (float)x.z, (float)B.radius[a]);
    } else if (t != AM_PLANE && B.root[a] >= 0) {
        int r0 = B.root[a];
        v3 x = ldv(N.cW + 3 * r0);
        c = make_float4((float)x.x, (float)x.y, (float)x.z, (float)N.r[r0]);
    }
    B.bc[a] = c;
}

void launch_broad_pack_subs(const DBodies& B, const DNodes& N, const int* subIds, int nsub, cudaStream_t s) {
    if (nsub <= 0) return;
    k_broad_pack_subs<<<(nsub + 255) / 256, 256, 0, s>>>(B, N, subIds, nsub);
    AM_LAUNCHED(1);
}

// True only when the FP32 distance proves the centres farther apart than the
// sum of the radii, i.e. when the exact FP64 quick exit would reject the pair
// too.  The margin, 1e-5 of the radii plus 1e-6 of the coordinates' size,
// covers the FP32 rounding of the centres, the differences and the sums
// (each below 2^-22 relative).
__device__ __forceinline__ bool far_apart32(float4 a, float4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    float d2 = dx * dx + dy * dy + dz * dz;
    float size = 1.f + fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(b.x) + fabsf(b.y) + fabsf(b.z);
    float T = (a.w + b.w) * 1.00001f + 1e-6f * size;
    return d2 > T * T;
}

// True only when the FP32 distance proves the centres closer than the sum of
// the radii, i.e. when the exact FP64 quick exit would accept the pair's
// geometry too (the same margin as far_apart32, on the other side).
__device__ __forceinline__ bool near32(float4 a, float4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    float d2 = dx * dx + dy * dy + dz * dz;
    float size = 1.f + fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(b.x) + fabsf(b.y) + fabsf(b.z);
    float T = (a.w + b.w) * 0.99999f - 1e-6f * size;
    return T > 0.f && d2 < T * T;
}

// the pair tests of pair_may_touch that come before the geometry
__device__ __forceinline__ bool pair_flags_allow(const DBodies& B, int a, int b) {
    int fa = B.flags[a], fb = B.flags[b];
    bool pa = fa & F_PINNED, pb = fb & F_PINNED;
    if (pa && pb) return false;
    return !((pa && (fb & F_SLEEPING)) || (pb && (fa & F_SLEEPING)));
}

// one warp per row i of the top-level list; ballot + popc keeps row-major order.
// With `masks`, the count pass stores every 32-pair chunk's hit mask (row i,
// chunk c at masks[i * mw + c]) and the emit pass reads them back instead of
// testing the pairs again.
template <bool WRITE>
__global__ void k_broad_rows(DBodies B, DNodes N, const int* top, int ntop, int* rowCount, const int* rowOff,
                             int* candA, int* candB, int cap, const int* topEnd, unsigned* masks, int mw) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= ntop - 1) return;
    int i = warp;
    int a = top[i];
    int run = WRITE ? rowOff[i] : 0;
    int end = topEnd ? topEnd[i] : ntop;   // batched scenes: pairs stay inside one scene
    const float4 ca = B.bc[a];
    unsigned* mrow = masks ? masks + (size_t)i * mw : nullptr;
    for (int j0 = i + 1; j0 < end; j0 += 32) {
        int j = j0 + lane;
        const int c = (j0 - i - 1) >> 5;
        bool hit = false;
        if (WRITE && mrow) {
            hit = (mrow[c] >> lane) & 1u;
        } else if (j < end) {
            int b = top[j];
            float4 cb = B.bc[b];
            // FP32 decides the geometry where its margin proves the FP64 quick
            // exit's answer (far: rejected, near: accepted); the band between
            // takes the exact test
            const bool prim = ca.w >= 0.f && cb.w >= 0.f;
            if (prim && far_apart32(ca, cb)) hit = false;
            else if (prim && near32(ca, cb)) hit = pair_flags_allow(B, a, b);
            else hit = pair_may_touch(B, N, a, b);
        }
        unsigned m = __ballot_sync(0xffffffffu, hit);
        if (!WRITE && mrow && lane == 0) mrow[c] = m;
        if (WRITE && hit) {
            int pos = run + __popc(m & ((1u << lane) - 1u));
            if (pos < cap) { candA[pos] = a; candB[pos] = top[j]; }
        }
        run += __popc(m);
    }
    if (!WRITE && lane == 0) rowCount[i] = run;
}

// candA == nullptr: the count pass (bounding-sphere pack, per-row counts,
// their scan into rowOff and dc->n_cand).  Otherwise the emit pass only, into
// the rows' offsets from the count pass of the same step.
int launch_broadphase(const DBodies& B, const DNodes& N, const int* top, int ntop, int* candA, int* candB,
                      int candCap, int* rowCount, int* rowOff, Scratch& sc, DCount* dc, cudaStream_t s,
                      const int* topEnd, unsigned* masks, int mw) {
    if (ntop < 2) {
        if (!candA) cudaMemsetAsync(&dc->n_cand, 0, sizeof(int), s);
        return 0;
    }
    int warps = ntop - 1;
    int blocks = (warps * 32 + 255) / 256;
    if (!candA) {
        k_broad_pack<<<(ntop + 127) / 128, 128, 0, s>>>(B, N, top, ntop);
        AM_LAUNCHED(1);
        k_broad_rows<false><<<blocks, 256, 0, s>>>(B, N, top, ntop, rowCount, nullptr, nullptr, nullptr, 0, topEnd,
                                                   masks, mw);
        AM_LAUNCHED(1);
        launch_scan(rowCount, rowOff, ntop - 1, sc, &dc->n_cand, s);
        return 0;
    }
    k_broad_rows<true><<<blocks, 256, 0, s>>>(B, N, top, ntop, nullptr, rowOff, candA, candB, candCap, topEnd,
                                              masks, mw);
    AM_LAUNCHED(1);
    return 0;
}

// ---------------------------------------------------------------------------
// collection expansion: candidate (A,B) -> sub-body pairs, A's bodies outer
__device__ __forceinline__ int nsub(const DBodies& B, const int* so, int x) {
    return (B.flags[x] & F_COLLECTION) ? (so[x + 1] - so[x]) : 1;
}
__device__ __forceinline__ int subat(const DBodies& B, const int* so, const int* si, int x, int k) {
    return (B.flags[x] & F_COLLECTION) ? si[so[x] + k] : x;
}

// A member pair of a collection's candidate is kept unless the FP32 bounds
// prove it apart (the first test of every collider would reject it: the
// broad phase's far_apart32 margin), so the kept pairs are the pairs that
// can touch, in the reference's order; a collection of m members then costs
// its touching member pairs instead of m times every body it may meet.
__device__ __forceinline__ bool sub_pair_kept(const DBodies& B, int a, int b) {
    const float4 ca = B.bc[a], cb = B.bc[b];
    return !(ca.w >= 0.f && cb.w >= 0.f && far_apart32(ca, cb));
}

__global__ void k_expand_count(DBodies B, const int* so, const int* si, const int* candA, const int* candB,
                               const DCount* dc, int* cnt) {
    int n = dc->n_cand;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int A = candA[i], Bb = candB[i];
        const int na = nsub(B, so, A), nb = nsub(B, so, Bb);
        if (na == 1 && nb == 1) { cnt[i] = 1; continue; }
        int k = 0;
        for (int p = 0; p < na; p++) {
            const int a = subat(B, so, si, A, p);
            for (int q = 0; q < nb; q++) k += sub_pair_kept(B, a, subat(B, so, si, Bb, q)) ? 1 : 0;
        }
        cnt[i] = k;
    }
}

__global__ void k_expand_write(DBodies B, const int* so, const int* si, const int* candA, const int* candB,
                               const DCount* dc, const int* off, DPairs P) {
    int n = dc->n_cand;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int A = candA[i], Bb = candB[i];
        const int na = nsub(B, so, A), nb = nsub(B, so, Bb);
        int o = off[i];
        if (na == 1 && nb == 1) {
            if (o < P.cap) { P.a[o] = A; P.b[o] = Bb; }
            continue;
        }
        for (int p = 0; p < na; p++) {
            const int a = subat(B, so, si, A, p);
            for (int q = 0; q < nb; q++) {
                const int b = subat(B, so, si, Bb, q);
                if (!sub_pair_kept(B, a, b)) continue;
                if (o < P.cap) { P.a[o] = a; P.b[o] = b; }
                o++;
            }
        }
    }
}

void launch_expand_pairs(const DBodies& B, const int* sub_off, const int* sub_ids, const int* candA,
                         const int* candB, int ncand, DPairs& P, Scratch& sc, DCount* dc, cudaStream_t s) {
    if (ncand <= 0) { cudaMemsetAsync(&dc->n_pairs, 0, sizeof(int), s); return; }
    k_expand_count<<<(ncand + 255) / 256, 256, 0, s>>>(B, sub_off, sub_ids, candA, candB, dc, sc.tmp);
    AM_LAUNCHED(1);
    launch_scan(sc.tmp, sc.tmp2, ncand, sc, &dc->n_pairs, s);
    k_expand_write<<<(ncand + 255) / 256, 256, 0, s>>>(B, sub_off, sub_ids, candA, candB, dc, sc.tmp2, P);
    AM_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
// Narrow phase colliders.  Each takes an emitter E(b1, b2, point, normal, bv1,
// bv2, info, violation) called in the reference's creation order.
struct CountEmit {
    int n;
    __device__ void operator()(int, int, v3, v3, int, int, int, double) { n++; }
};

struct WriteEmit {
    const DBodies* B;
    DContacts* C;
    int base, k, pair;
    int* overflow;
    __device__ void operator()(int b1, int b2, v3 pW, v3 nW, int bv1, int bv2, int info, double cv);
};

// Contact.set + computeJacobian(false, ...) (Contact.java:159-255)
__device__ void WriteEmit::operator()(int b1, int b2, v3 pW, v3 nW, int bv1, int bv2, int info, double cv) {
    int c = base + k;
    k++;
    int cap = C->cap;
    if (c >= cap) { *overflow = 1; return; }
    const DBodies& Bd = *B;
    C->b1[c] = b1; C->b2[c] = b2; C->bv1[c] = bv1; C->bv2[c] = bv2; C->info[c] = info; C->pair[c] = pair;
    C->state[c] = AM_STATE_CLEAR; C->fresh[c] = 1;
    C->cv[c] = cv; C->pcv[c] = 0.0;
    for (int r = 0; r < 3; r++) { C->lam[r * cap + c] = 0.0; C->lamw[r * cap + c] = 0.0; }
    for (int r = 0; r < 6; r++) C->bD[r * cap + c] = 0.0;
    double anx = fabs(nW.x), any = fabs(nW.y), anz = fabs(nW.z);
    v3 t1;
    if (anx < any && anx < anz) t1 = mk(1, 0, 0);
    else if (any < anz) t1 = mk(0, 1, 0);
    else t1 = mk(0, 0, 1);
    v3 t2 = cross(nW, t1);
    normalize(t2);
    t1 = cross(t2, nW);
    int s1 = Bd.parent[b1] >= 0 ? Bd.parent[b1] : b1;
    int s2 = Bd.parent[b2] >= 0 ? Bd.parent[b2] : b2;
    C->sb1[c] = s1; C->sb2[c] = s2;
    v3 r1 = sub(pW, bodyX(Bd, s1));
    v3 r2 = sub(pW, bodyX(Bd, s2));
    v3 rows[12];
    rows[0] = scale(-1, nW);  rows[1] = cross(nW, r1);  rows[2] = nW;  rows[3] = cross(r2, nW);
    rows[4] = scale(-1, t1);  rows[5] = cross(t1, r1);  rows[6] = t1;  rows[7] = cross(r2, t1);
    rows[8] = scale(-1, t2);  rows[9] = cross(t2, r1);  rows[10] = t2; rows[11] = cross(r2, t2);
    for (int q = 0; q < 12; q++) {
        C->J[(3 * q + 0) * cap + c] = rows[q].x;
        C->J[(3 * q + 1) * cap + c] = rows[q].y;
        C->J[(3 * q + 2) * cap + c] = rows[q].z;
    }
    m3 R1 = bodyR(Bd, b1);
    v3 x1 = bodyX(Bd, b1);
    v3 fr[4] = {tinvpoint(R1, x1, pW), mtxv(R1, nW), mtxv(R1, t1), mtxv(R1, t2)};
    for (int q = 0; q < 4; q++) {
        C->f[(3 * q + 0) * cap + c] = fr[q].x;
        C->f[(3 * q + 1) * cap + c] = fr[q].y;
        C->f[(3 * q + 2) * cap + c] = fr[q].z;
    }
}

__device__ __forceinline__ v3 corner(v3 p, int k) {  // +++ ++- +-+ +-- -++ -+- --+ ---
    return mk((k & 4) ? -p.x : p.x, (k & 2) ? -p.y : p.y, (k & 1) ? -p.z : p.z);
}

// BoxPlane.dBoxPlane (collision/BoxPlane.java:27-52); the plane is body 1
template <class E>
__device__ void box_plane(const DBodies& B, int box, int pl, E& emit) {
    v3 n = ldv(B.plane + 4 * pl);
    double d = B.plane[4 * pl + 3];
    v3 x = bodyX(B, box);
    if (x.x * n.x + x.y * n.y + x.z * n.z + d > B.radius[box]) return;
    v3 p = scale(0.5, ldv(B.size + 3 * box));
    m3 R = bodyR(B, box);
    for (int k = 0; k < 8; k++) {
        v3 q = tpoint(R, x, corner(p, k));
        double s = q.x * n.x + q.y * n.y + q.z * n.z + d;
        if (s < 0) emit(pl, box, q, n, AM_BV_NULL, AM_BV_NULL, k, s);
    }
}

// BoxSphere.dBoxSphereTest (collision/BoxSphere.java:156-233)
__device__ bool box_sphere_test(const DBodies& B, int box, v3 c, double r) {
    v3 x = bodyX(B, box);
    if (dist(c, x) > B.radius[box] + r) return false;
    v3 p = scale(0.5, ldv(B.size + 3 * box));
    v3 cB = tinvpoint(bodyR(B, box), x, c);
    if (cB.x - p.x > r) return false;
    if (-p.x - cB.x > r) return false;
    if (cB.y - p.y > r) return false;
    if (-p.y - cB.y > r) return false;
    if (cB.z - p.z > r) return false;
    if (-p.z - cB.z > r) return false;
    for (int k = 0; k < 8; k++)
        if (dist(cB, corner(p, k)) - r < 0) return true;
    if (-p.x <= cB.x && cB.x <= p.x) {
        if (cB.y >= p.y && cB.z >= p.z) { if (length(mk(0, cB.y - p.y, cB.z - p.z)) - r < 0) return true; }
        else if (cB.y <= -p.y && cB.z >= p.z) { if (length(mk(0, cB.y + p.y, cB.z - p.z)) - r < 0) return true; }
        else if (cB.y >= p.y && cB.z <= -p.z) { if (length(mk(0, cB.y - p.y, cB.z + p.z)) - r < 0) return true; }
        else if (cB.y <= -p.y && cB.z <= -p.z) { if (length(mk(0, cB.y + p.y, cB.z + p.z)) - r < 0) return true; }
    }
    if (-p.y <= cB.y && cB.y <= p.y) {
        if (cB.x >= p.x && cB.z >= p.z) { if (length(mk(cB.x - p.x, 0, cB.z - p.z)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.z >= p.z) { if (length(mk(cB.x + p.x, 0, cB.z - p.z)) - r < 0) return true; }
        else if (cB.x >= p.x && cB.z <= -p.z) { if (length(mk(cB.x - p.x, 0, cB.z + p.z)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.z <= -p.z) { if (length(mk(cB.x + p.x, 0, cB.z + p.z)) - r < 0) return true; }
    }
    if (-p.z < cB.z && cB.z < p.z) {
        if (cB.x >= p.x && cB.y >= p.y) { if (length(mk(cB.x - p.x, cB.y - p.y, 0)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.y >= p.y) { if (length(mk(cB.x + p.x, cB.y - p.y, 0)) - r < 0) return true; }
        else if (cB.x >= p.x && cB.y <= -p.y) { if (length(mk(cB.x - p.x, cB.y + p.y, 0)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.y <= -p.y) { if (length(mk(cB.x + p.x, cB.y + p.y, 0)) - r < 0) return true; }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.y <= cB.y && cB.y <= p.y) {
        if (cB.z > 0) { if (cB.z - p.z - r < 0) return true; }
        else { if (-p.z - cB.z - r < 0) return true; }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.y > 0) { if (cB.y - p.y - r < 0) return true; }
        else { if (-p.y - cB.y - r < 0) return true; }
    }
    if (-p.y <= cB.y && cB.y <= p.y && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.x > 0) { if (cB.x - p.x - r < 0) return true; }
        else { if (-p.x - cB.x - r < 0) return true; }
    }
    return false;
}

// BoxSphere.dBoxSphere with test1 / test2 (collision/BoxSphere.java:58-144, 242-275)
template <class E>
__device__ void box_sphere(const DBodies& B, int box, int sph, v3 c, double r, E& emit) {
    v3 x = bodyX(B, box);
    m3 R = bodyR(B, box);
    v3 p = scale(0.5, ldv(B.size + 3 * box));
    v3 cB = tinvpoint(R, x, c);
    double depth = 1;
    v3 pos = mk(0, 0, 0), nrm = mk(0, 0, 0);
    for (int k = 0; k < 8; k++) {
        v3 q = corner(p, k);
        double s = dist(cB, q) - r;
        if (s > 0) continue;
        if (s < depth) { pos = q; nrm = sub(cB, q); normalize(nrm); depth = s; }
    }
#define T2(S, PX, PY, PZ, NX, NY, NZ)                                              \
    {                                                                             \
        double s_ = (S);                                                          \
        if (!(s_ > 0) && s_ < depth) { pos = mk(PX, PY, PZ); nrm = mk(NX, NY, NZ); depth = s_; } \
    }
    double s;
    v3 v;
    if (-p.x <= cB.x && cB.x <= p.x) {
        if (cB.y >= p.y && cB.z >= p.z) { v = mk(0, cB.y - p.y, cB.z - p.z); s = length(v); s -= r; T2(s, cB.x, p.y, p.z, v.x, v.y, v.z); }
        else if (cB.y <= -p.y && cB.z >= p.z) { v = mk(0, cB.y + p.y, cB.z - p.z); s = length(v); s -= r; T2(s, cB.x, -p.y, p.z, v.x, v.y, v.z); }
        else if (cB.y >= p.y && cB.z <= -p.z) { v = mk(0, cB.y - p.y, cB.z + p.z); s = length(v); s -= r; T2(s, cB.x, p.y, -p.z, v.x, v.y, v.z); }
        else if (cB.y <= -p.y && cB.z <= -p.z) { v = mk(0, cB.y + p.y, cB.z + p.z); s = length(v); s -= r; T2(s, cB.x, -p.y, -p.z, v.x, v.y, v.z); }
    }
    if (-p.y <= cB.y && cB.y <= p.y) {
        if (cB.x >= p.x && cB.z >= p.z) { v = mk(cB.x - p.x, 0, cB.z - p.z); s = length(v); s -= r; T2(s, p.x, cB.y, p.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.z >= p.z) { v = mk(cB.x + p.x, 0, cB.z - p.z); s = length(v); s -= r; T2(s, -p.x, cB.y, p.z, v.x, v.y, v.z); }
        else if (cB.x >= p.x && cB.z <= -p.z) { v = mk(cB.x - p.x, 0, cB.z + p.z); s = length(v); s -= r; T2(s, p.x, cB.y, -p.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.z <= -p.z) { v = mk(cB.x + p.x, 0, cB.z + p.z); s = length(v); s -= r; T2(s, -p.x, cB.y, -p.z, v.x, v.y, v.z); }
    }
    if (-p.z <= cB.z && cB.z <= p.z) {
        if (cB.x >= p.x && cB.y >= p.y) { v = mk(cB.x - p.x, cB.y - p.y, 0); s = length(v); s -= r; T2(s, p.x, p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.y >= p.y) { v = mk(cB.x + p.x, cB.y - p.y, 0); s = length(v); s -= r; T2(s, -p.x, p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x >= p.x && cB.y <= -p.y) { v = mk(cB.x - p.x, cB.y + p.y, 0); s = length(v); s -= r; T2(s, p.x, -p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.y <= -p.y) { v = mk(cB.x + p.x, cB.y + p.y, 0); s = length(v); s -= r; T2(s, -p.x, -p.y, cB.z, v.x, v.y, v.z); }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.y <= cB.y && cB.y <= p.y) {
        if (cB.z > 0) { s = cB.z - p.z - r; T2(s, cB.x, cB.y, p.z, 0, 0, 1); }
        else { s = -p.z - cB.z - r; T2(s, cB.x, cB.y, -p.z, 0, 0, -1); }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.y > 0) { s = cB.y - p.y - r; T2(s, cB.x, p.y, cB.z, 0, 1, 0); }
        else { s = -p.y - cB.y - r; T2(s, cB.x, -p.y, cB.z, 0, -1, 0); }
    }
    if (-p.y <= cB.y && cB.y <= p.y && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.x > 0) { s = cB.x - p.x - r; T2(s, p.x, cB.y, cB.z, 1, 0, 0); }
        else { s = -p.x - cB.x - r; T2(s, -p.x, cB.y, cB.z, -1, 0, 0); }
    }
#undef T2
    if (depth != 1) {
        pos = tpoint(R, x, pos);
        nrm = mxv(R, nrm);
        normalize(nrm);
        emit(box, sph, pos, nrm, AM_BV_NULL, AM_BV_NULL, 0, depth);
    }
}

// intersectRectQuad (collision/BoxBox.java:140-209): clip the incident quad
// against the reference rectangle; ping-pong between ret and a local buffer.
__device__ int clip_rect_quad(const double h[2], const double quad[8], double ret[16]) {
    double buffer[16];
    const double* q = quad;
    double* r = ret;
    int nq = 4, nr = 0;
    bool qIsRet = false;
    for (int dir = 0; dir <= 1; dir++) {
        for (int sign = -1; sign <= 1; sign += 2) {
            int pq = 0, pr = 0;
            nr = 0;
            double sg = (double)sign;
            for (int i = nq; i > 0; i--) {
                if (sg * q[pq + dir] < h[dir]) {
                    r[pr] = q[pq];
                    r[pr + 1] = q[pq + 1];
                    pr += 2;
                    nr++;
                    if (nr & 8) { q = r; qIsRet = (r == ret); goto done; }
                }
                int nx = (i > 1) ? pq + 2 : 0;
                if ((sg * q[pq + dir] < h[dir]) ^ (sg * q[nx + dir] < h[dir])) {
                    r[pr + 1 - dir] = q[pq + 1 - dir] +
                                      (q[nx + 1 - dir] - q[pq + 1 - dir]) / (q[nx + dir] - q[pq + dir]) *
                                          (sg * h[dir] - q[pq + dir]);
                    r[pr + dir] = sg * h[dir];
                    pr += 2;
                    nr++;
                    if (nr & 8) { q = r; qIsRet = (r == ret); goto done; }
                }
                pq += 2;
            }
            q = r;
            qIsRet = (q == ret);
            r = qIsRet ? buffer : ret;
            nq = nr;
        }
    }
done:
    if (!qIsRet)
        for (int k = 0; k < 2 * nr; k++) ret[k] = q[k];
    return nr;
}

// BoxBox.dBoxBox (collision/BoxBox.java:433-859), ODE's separating-axis test
template <class E>
__device__ void box_box(const DBodies& B, int b1, int b2, E& emit) {
    v3 p1 = bodyX(B, b1), p2 = bodyX(B, b2);
    v3 p = sub(p2, p1);
    if (length(p) > B.radius[b1] + B.radius[b2]) return;
    m3 R1 = bodyR(B, b1), R2 = bodyR(B, b2);
    v3 pp = mtxv(R1, p);
    v3 A = scale(0.5, ldv(B.size + 3 * b1));
    v3 Bh = scale(0.5, ldv(B.size + 3 * b2));
    double Rm[3][3], Q[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { Rm[i][j] = dot(col(R1, i), col(R2, j)); Q[i][j] = fabs(Rm[i][j]); }
    double R11 = Rm[0][0], R12 = Rm[0][1], R13 = Rm[0][2], R21 = Rm[1][0], R22 = Rm[1][1], R23 = Rm[1][2];
    double R31 = Rm[2][0], R32 = Rm[2][1], R33 = Rm[2][2];
    double Q11 = Q[0][0], Q12 = Q[0][1], Q13 = Q[0][2], Q21 = Q[1][0], Q22 = Q[1][1], Q23 = Q[1][2];
    double Q31 = Q[2][0], Q32 = Q[2][1], Q33 = Q[2][2];
    double s = -INFINITY;
    bool invert = false;
    int code = 0, nMat = -1, nCol = 0;   // nMat: 1 -> R1 column, 2 -> R2 column, -1 -> normalC
    v3 normalC = mk(0, 0, 0);
    const double tiny = 1e-5, fudge = 1.05;
#define TST1(E1, E2, MAT, COL, CC)                                                                  \
    {                                                                                              \
        double e1_ = (E1);                                                                          \
        double s2_ = fabs(e1_) - (E2);                                                              \
        if (s2_ > 0) return;                                                                        \
        if (s2_ > s + tiny) { s = s2_; nMat = MAT; nCol = COL; invert = e1_ < 0; code = CC; }        \
    }
#define TST2(E1, E2, N1, N2, N3, CC)                                                                \
    {                                                                                              \
        double e1_ = (E1);                                                                          \
        double s2_ = fabs(e1_) - (E2);                                                              \
        if (s2_ > 0) return;                                                                        \
        double n1_ = (N1), n2_ = (N2), n3_ = (N3);                                                  \
        double l_ = sqrt(n1_ * n1_ + n2_ * n2_ + n3_ * n3_);                                        \
        if (l_ > 0) {                                                                              \
            s2_ /= l_;                                                                              \
            if (s2_ * fudge > s) { s = s2_; nMat = -1; nCol = 0; normalC = mk(n1_ / l_, n2_ / l_, n3_ / l_); invert = e1_ < 0; code = CC; } \
        }                                                                                          \
    }
    TST1(pp.x, A.x + Bh.x * Q11 + Bh.y * Q12 + Bh.z * Q13, 1, 0, 1);
    TST1(pp.y, A.y + Bh.x * Q21 + Bh.y * Q22 + Bh.z * Q23, 1, 1, 2);
    TST1(pp.z, A.z + Bh.x * Q31 + Bh.y * Q32 + Bh.z * Q33, 1, 2, 3);
    TST1(dot(col(R2, 0), p), A.x * Q11 + A.y * Q21 + A.z * Q31 + Bh.x, 2, 0, 4);
    TST1(dot(col(R2, 1), p), A.x * Q12 + A.y * Q22 + A.z * Q32 + Bh.y, 2, 1, 5);
    TST1(dot(col(R2, 2), p), A.x * Q13 + A.y * Q23 + A.z * Q33 + Bh.z, 2, 2, 6);
    TST2(pp.z * R21 - pp.y * R31, A.y * Q31 + A.z * Q21 + Bh.y * Q13 + Bh.z * Q12, 0, -R31, R21, 7);
    TST2(pp.z * R22 - pp.y * R32, A.y * Q32 + A.z * Q22 + Bh.x * Q13 + Bh.z * Q11, 0, -R32, R22, 8);
    TST2(pp.z * R23 - pp.y * R33, A.y * Q33 + A.z * Q23 + Bh.x * Q12 + Bh.y * Q11, 0, -R33, R23, 9);
    TST2(pp.x * R31 - pp.z * R11, A.x * Q31 + A.z * Q11 + Bh.y * Q23 + Bh.z * Q22, R31, 0, -R11, 10);
    TST2(pp.x * R32 - pp.z * R12, A.x * Q32 + A.z * Q12 + Bh.x * Q23 + Bh.z * Q21, R32, 0, -R12, 11);
    TST2(pp.x * R33 - pp.z * R13, A.x * Q33 + A.z * Q13 + Bh.x * Q22 + Bh.y * Q21, R33, 0, -R13, 12);
    TST2(pp.y * R11 - pp.x * R21, A.x * Q21 + A.y * Q11 + Bh.y * Q33 + Bh.z * Q32, -R21, R11, 0, 13);
    TST2(pp.y * R12 - pp.x * R22, A.x * Q22 + A.y * Q12 + Bh.x * Q33 + Bh.z * Q31, -R22, R12, 0, 14);
    TST2(pp.y * R13 - pp.x * R23, A.x * Q23 + A.y * Q13 + Bh.x * Q32 + Bh.y * Q31, -R23, R13, 0, 15);
#undef TST1
#undef TST2
    if (code == 0) return;
    v3 normal = nMat == 1 ? col(R1, nCol) : (nMat == 2 ? col(R2, nCol) : mxv(R1, normalC));
    if (invert) { normal.x *= -1; normal.y *= -1; normal.z *= -1; }
    double depth = -s;
    int info = 0;
    if (code > 6) {   // edge-edge
        v3 pa = p1;
        for (int j = 0; j < 3; j++) {
            double sign = (dot(normal, col(R1, j)) > 0) ? 1.0 : -1.0;
            pa.x += sign * comp(A, j) * R1.m[j];
            pa.y += sign * comp(A, j) * R1.m[3 + j];
            pa.z += sign * comp(A, j) * R1.m[6 + j];
        }
        v3 pb = p2;
        for (int j = 0; j < 3; j++) {
            double sign = (dot(normal, col(R2, j)) > 0) ? -1.0 : 1.0;
            pb.x += sign * comp(Bh, j) * R2.m[j];
            pb.y += sign * comp(Bh, j) * R2.m[3 + j];
            pb.z += sign * comp(Bh, j) * R2.m[6 + j];
        }
        v3 ua = col(R1, (code - 7) / 3);
        v3 ub = col(R2, (code - 7) % 3);
        v3 q = sub(pb, pa);     // dLineClosestApproach (BoxBox.java:366-383)
        double uaub = dot(ua, ub);
        double q1 = dot(ua, q);
        double q2 = -dot(ub, q);
        double d = 1 - uaub * uaub;
        double alpha, beta;
        if (d <= 0.0001) { alpha = 0; beta = 0; }
        else { d = 1.0 / d; alpha = (q1 + uaub * q2) * d; beta = (uaub * q1 + q2) * d; }
        pa = scaleadd(alpha, ua, pa);
        pb = scaleadd(beta, ub, pb);
        v3 pos = add(pa, pb);
        pos.x *= 0.5; pos.y *= 0.5; pos.z *= 0.5;
        emit(b1, b2, pos, normal, AM_BV_NULL, AM_BV_NULL, info++, -depth);
        return;
    }
    bool fa = code <= 3;
    m3 Ra = fa ? R1 : R2, Rb = fa ? R2 : R1;
    v3 pa = fa ? p1 : p2, pb = fa ? p2 : p1, Sa = fa ? A : Bh, Sb = fa ? Bh : A;
    v3 normal2 = fa ? normal : scale(-1, normal);
    v3 nr = mtxv(Rb, normal2);
    v3 anr = mk(fabs(nr.x), fabs(nr.y), fabs(nr.z));
    int lanr, a1, a2;
    if (anr.y > anr.x) {
        if (anr.y > anr.z) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr.x > anr.z) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    v3 center;
    if (comp(nr, lanr) < 0) {
        for (int i = 0; i < 3; i++) setc(center, i, comp(pb, i) - comp(pa, i) + comp(Sb, lanr) * Rb.m[3 * i + lanr]);
    } else {
        for (int i = 0; i < 3; i++) setc(center, i, comp(pb, i) - comp(pa, i) - comp(Sb, lanr) * Rb.m[3 * i + lanr]);
    }
    int codeN = fa ? code - 1 : code - 4;
    int code1, code2;
    if (codeN == 0) { code1 = 1; code2 = 2; }
    else if (codeN == 1) { code1 = 0; code2 = 2; }
    else { code1 = 0; code2 = 1; }
    double c1 = dot(center, col(Ra, code1));
    double c2 = dot(center, col(Ra, code2));
    double m11 = dot(col(Ra, code1), col(Rb, a1));
    double m12 = dot(col(Ra, code1), col(Rb, a2));
    double m21 = dot(col(Ra, code2), col(Rb, a1));
    double m22 = dot(col(Ra, code2), col(Rb, a2));
    double quad[8];
    {
        double k1 = m11 * comp(Sb, a1), k2 = m21 * comp(Sb, a1), k3 = m12 * comp(Sb, a2), k4 = m22 * comp(Sb, a2);
        quad[0] = c1 - k1 - k3; quad[1] = c2 - k2 - k4;
        quad[2] = c1 - k1 + k3; quad[3] = c2 - k2 + k4;
        quad[4] = c1 + k1 + k3; quad[5] = c2 + k2 + k4;
        quad[6] = c1 + k1 - k3; quad[7] = c2 + k2 - k4;
    }
    double rect[2] = {comp(Sa, code1), comp(Sa, code2)};
    double ret[16];
    int n = clip_rect_quad(rect, quad, ret);
    if (n < 1) return;
    double det1 = 1.0 / (m11 * m22 - m12 * m21);
    m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
    double point[24], dep[8];
    int cnum = 0;
    for (int j = 0; j < n; j++) {
        double k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        double k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (int i = 0; i < 3; i++) point[cnum * 3 + i] = comp(center, i) + k1 * Rb.m[3 * i + a1] + k2 * Rb.m[3 * i + a2];
        dep[cnum] = comp(Sa, codeN) - (normal2.x * point[cnum * 3] + normal2.y * point[cnum * 3 + 1] + normal2.z * point[cnum * 3 + 2]);
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    for (int j = 0; j < cnum; j++) {
        v3 pos = mk(point[j * 3] + pa.x, point[j * 3 + 1] + pa.y, point[j * 3 + 2] + pa.z);
        emit(b1, b2, pos, normal, AM_BV_NULL, AM_BV_NULL, info++, -dep[j]);
    }
}

// Sphere-tree traversals with an explicit stack (children pushed in reverse
// so they pop in index order, matching the recursive reference).
// Depth-first traversal stacks of the tree colliders.  A stack holds, for
// each descent on the current path, the siblings still to visit, so it needs
// at most (descents on a path) x (largest child count - 1) + 1 entries: for
// two trees of depth 3 whose nodes have up to 30 children (the reference's
// .sph hierarchies), 6 x 29 + 1 = 175.  A deeper need raises AM_E_CAPACITY.
static const int STACK = 192;

// collideSphereTreeAndPlane (CollisionProcessor.java:793-826); tree body is body 1
template <class E>
__device__ void tree_plane(const DBodies& B, const DNodes& N, int root, int body, int pl, E& emit, int* err) {
    v3 n = ldv(B.plane + 4 * pl);
    double pd = B.plane[4 * pl + 3];
    v3 pp = ldv(B.pp + 3 * pl);
    int st[STACK];
    int sp = 0;
    st[sp++] = root;
    while (sp) {
        int k = st[--sp];
        v3 c = ldv(N.cW + 3 * k);
        double d = n.x * c.x + n.y * c.y + n.z * c.z + pd - N.r[k];
        if (!(d < 0)) continue;
        int c0 = N.child0[k], nc = N.nchild[k];
        if (c0 < 0) {
            v3 t = sub(c, pp);
            double val = dot(t, n);
            t = scale(val, n);
            v3 cw = sub(c, t);
            emit(body, pl, cw, scale(-1, n), k, AM_BV_PLANE(pl), 0, d);
        } else {
            if (sp + nc > STACK) { *err = AM_E_CAPACITY; return; }
            for (int q = nc - 1; q >= 0; q--) st[sp++] = c0 + q;
        }
    }
}

// collideBoxAndSphereTree (CollisionProcessor.java:837-850); box is body 1
template <class E>
__device__ void box_tree(const DBodies& B, const DNodes& N, int root, int box, int tree, E& emit, int* err) {
    int st[STACK];
    int sp = 0;
    st[sp++] = root;
    while (sp) {
        int k = st[--sp];
        v3 c = ldv(N.cW + 3 * k);
        double r = N.r[k];
        if (!box_sphere_test(B, box, c, r)) continue;
        int c0 = N.child0[k], nc = N.nchild[k];
        if (c0 >= 0) {
            if (sp + nc > STACK) { *err = AM_E_CAPACITY; return; }
            for (int q = nc - 1; q >= 0; q--) st[sp++] = c0 + q;
        } else {
            box_sphere(B, box, tree, c, r, emit);
        }
    }
}

// collideSphereTrees + processCollision (CollisionProcessor.java:975-1009, 1036-1056)
template <class E>
__device__ void tree_tree(const DBodies& B, const DNodes& N, int r1, int r2, int b1, int b2, E& emit, int* err) {
    int s1[STACK], s2[STACK];
    int sp = 0;
    s1[sp] = r1; s2[sp] = r2; sp++;
    while (sp) {
        sp--;
        int i1 = s1[sp], i2 = s2[sp];
        v3 c1 = ldv(N.cW + 3 * i1), c2 = ldv(N.cW + 3 * i2);
        double ra = N.r[i1], rb = N.r[i2];
        if (!(dist2(c1, c2) < (ra + rb) * (ra + rb))) continue;
        bool l1 = N.child0[i1] < 0, l2 = N.child0[i2] < 0;
        if (l1 && l2) {
            double distance = dist(c1, c2);
            double dbc = rb + ra;
            if (distance < dbc) {
                double alpha = (ra - rb + distance) / (2 * distance);
                v3 cw = mk((1 - alpha) * c1.x + alpha * c2.x, (1 - alpha) * c1.y + alpha * c2.y,
                           (1 - alpha) * c1.z + alpha * c2.z);
                v3 nrm = sub(c2, c1);
                normalize(nrm);
                emit(b1, b2, cw, nrm, i1, i2, 0, distance - dbc);
            }
            continue;
        }
        bool down2 = l1 || (!l2 && ra <= rb);
        int par = down2 ? i2 : i1;
        int c0 = N.child0[par], nc = N.nchild[par];
        if (sp + nc > STACK) { *err = AM_E_CAPACITY; return; }
        for (int q = nc - 1; q >= 0; q--) {
            s1[sp] = down2 ? i1 : c0 + q;
            s2[sp] = down2 ? c0 + q : i2;
            sp++;
        }
    }
}

// CollisionProcessor.narrowPhase dispatch for two primitive bodies
template <class E>
__device__ void narrow_pair(const DBodies& B, const DNodes& N, int b1, int b2, E& emit, int* err) {
    int t1 = B.type[b1], t2 = B.type[b2];
    if (t1 == AM_PLANE) {
        if (t2 == AM_PLANE) return;
        if (t2 == AM_BOX) box_plane(B, b2, b1, emit);
        else tree_plane(B, N, B.root[b2], b2, b1, emit, err);
    } else if (t1 == AM_BOX) {
        if (t2 == AM_PLANE) box_plane(B, b1, b2, emit);
        else if (t2 == AM_BOX) box_box(B, b1, b2, emit);
        else box_tree(B, N, B.root[b2], b1, b2, emit, err);
    } else {
        if (t2 == AM_PLANE) tree_plane(B, N, B.root[b1], b1, b2, emit, err);
        else if (t2 == AM_BOX) box_tree(B, N, B.root[b1], b2, b1, emit, err);
        else tree_tree(B, N, B.root[b1], B.root[b2], b1, b2, emit, err);
    }
}

// body-type class of a pair: 0 box-plane, 1 sphere tree on plane, 2 box-box,
// 3 box-tree, 4 tree-tree (planes never pair with planes)
__device__ __forceinline__ int pair_class(const DBodies& B, int b1, int b2) {
    int t1 = B.type[b1], t2 = B.type[b2];
    if (t1 == AM_PLANE || t2 == AM_PLANE) return (t1 == AM_BOX || t2 == AM_BOX) ? 0 : 1;
    if (t1 == AM_BOX && t2 == AM_BOX) return 2;
    return (t1 == AM_BOX || t2 == AM_BOX) ? 3 : 4;
}

// class counts (warp-aggregated atomics into cls[0..4])
__global__ void k_pair_class_count(DBodies B, DPairs P, int n, int* cls) {
    const unsigned FULL = 0xffffffffu;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        int c = i < n ? pair_class(B, P.a[i], P.b[i]) : -1;
        for (int k = 0; k < 5; k++) {
            unsigned m = __ballot_sync(FULL, c == k);
            if (m && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&cls[k], __popc(m));
        }
    }
}

// positions: each class starts after the smaller classes; within a class the
// order is arbitrary (every pair writes its own outputs)
__global__ void k_pair_perm(DBodies B, DPairs P, int n, int* cls) {
    const unsigned FULL = 0xffffffffu;
    __shared__ int s_off[5];
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < 5; k++) { s_off[k] = run; run += cls[k]; }
    }
    __syncthreads();
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        int c = i < n ? pair_class(B, P.a[i], P.b[i]) : -1;
        const int lane = threadIdx.x & 31;
        for (int k = 0; k < 5; k++) {
            unsigned m = __ballot_sync(FULL, c == k);
            if (!m) continue;
            int leader = __ffs(m) - 1, pos = 0;
            if (lane == leader) pos = atomicAdd(&cls[5 + k], __popc(m));
            pos = __shfl_sync(FULL, pos, leader);
            if (c == k) P.perm[s_off[k] + pos + __popc(m & ((1u << lane) - 1))] = i;
        }
    }
}

void launch_pair_order(const DBodies& B, DPairs& P, int n, int* cls, cudaStream_t s) {
    cudaMemsetAsync(cls, 0, sizeof(int) * 16, s);
    int blocks = std::min((n + 255) / 256, 4 * 152);
    k_pair_class_count<<<blocks, 256, 0, s>>>(B, P, n, cls);
    k_pair_perm<<<blocks, 256, 0, s>>>(B, P, n, cls);
    AM_LAUNCHED(2);
}

__global__ void k_narrow_count(DBodies B, DNodes N, DPairs P, DCount* dc) {
    int n = dc->n_pairs;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = P.perm[j];
        CountEmit e{0};
        int err = 0;
        narrow_pair(B, N, P.a[i], P.b[i], e, &err);
        if (err) dc->error = err;
        P.count[i] = e.n;
    }
}

__global__ void k_narrow_emit(DBodies B, DNodes N, DPairs P, DContacts C, DCount* dc) {
    int n = dc->n_pairs;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = P.perm[j];
        WriteEmit e{&B, &C, P.off[i], 0, i, &dc->overflow};
        int err = 0;
        narrow_pair(B, N, P.a[i], P.b[i], e, &err);
        if (err) dc->error = err;
    }
}

// Staged narrow phase (one collider pass): when no pair can yield more than
// NSTAGE contacts (boxes, planes and single-sphere trees), the record pass
// runs the colliders once, counting and keeping each pair's raw contacts
// (point, normal, depth, BV ids, info, bodies) in emission order; after the
// scan the set pass writes Contact.set for them at the pair's offset.  The
// result is the two-pass result: the same emitter arguments in the same
// order.  A pair that yields more than NSTAGE raises *stageOvf, and the step
// falls back to the emit pass.
static const int NSTAGE = 8;
struct StageEmit {
    double* sd;      // 7 doubles per staged contact: point, normal, depth
    int* si;         // 5 ints: body1, body2, bv1, bv2, info
    int base, n;
    int* ovf;
    __device__ void operator()(int b1, int b2, v3 pW, v3 nW, int bv1, int bv2, int info, double cv) {
        if (n < NSTAGE) {
            size_t q = (size_t)base * NSTAGE + n;
            double* d = sd + 7 * q;
            d[0] = pW.x; d[1] = pW.y; d[2] = pW.z; d[3] = nW.x; d[4] = nW.y; d[5] = nW.z; d[6] = cv;
            int* e = si + 5 * q;
            e[0] = b1; e[1] = b2; e[2] = bv1; e[3] = bv2; e[4] = info;
        } else {
            *ovf = 1;
        }
        n++;
    }
};

__global__ void k_narrow_record(DBodies B, DNodes N, DPairs P, DCount* dc, double* sd, int* si, int* ovf) {
    int n = dc->n_pairs;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = P.perm[j];
        StageEmit e{sd, si, i, 0, ovf};
        int err = 0;
        narrow_pair(B, N, P.a[i], P.b[i], e, &err);
        if (err) dc->error = err;
        P.count[i] = e.n;
    }
}

__global__ void k_narrow_set(DBodies B, DPairs P, DContacts C, DCount* dc, const double* sd, const int* si) {
    int n = dc->n_pairs;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = P.perm[j];
        WriteEmit e{&B, &C, P.off[i], 0, i, &dc->overflow};
        const int cnt = P.count[i];
        for (int k = 0; k < cnt; k++) {
            size_t q = (size_t)i * NSTAGE + k;
            const double* d = sd + 7 * q;
            const int* x = si + 5 * q;
            e(x[0], x[1], mk(d[0], d[1], d[2]), mk(d[3], d[4], d[5]), x[2], x[3], x[4], d[6]);
        }
    }
}

int narrow_stage_slots() { return NSTAGE; }

void launch_narrow(const DBodies& B, const DNodes& N, DPairs& P, DContacts& C, Scratch& sc, DCount* dc,
                   bool emit, cudaStream_t s, double* sd, int* si, int* ovf) {
    (void)sc;
    if (sd) {
        if (!emit) k_narrow_record<<<4 * 152, 128, 0, s>>>(B, N, P, dc, sd, si, ovf);
        else k_narrow_set<<<4 * 152, 128, 0, s>>>(B, P, C, dc, sd, si);
    } else {
        if (!emit) k_narrow_count<<<4 * 152, 128, 0, s>>>(B, N, P, dc);
        else k_narrow_emit<<<4 * 152, 128, 0, s>>>(B, N, P, C, dc);
    }
    AM_LAUNCHED(1);
}

}  // namespace am
