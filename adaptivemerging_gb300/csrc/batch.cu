// batch.cu -- many independent scenes solved by one launch.
//
// The scenes' bodies are concatenated (scene s owns body slots
// [sceneBodyOff[s], sceneBodyOff[s+1])); the collision pipeline runs on the
// whole batch with the broad phase restricted to pairs inside one scene, so
// every scene's contacts and body-pair groups are contiguous runs.  The solve
// then runs one CTA per scene:
//   * the scene's body-pair groups are coloured inside the CTA (first-fit
//     Jones-Plassmann over scene-local bodies; 3-4 colours for a bin);
//   * every contact is packed into a 64-float record (J, jinv J.w for both
//     bodies, b, D, 1/(D + c), mu), stored in colour order ("slots"), so a
//     colour's records form one contiguous run;
//   * the scene's delta-v lives in shared memory (FP32) for the whole solve;
//     the records and multipliers of a scene that fits the staging buffer
//     are loaded into shared memory once and stay there; a larger scene is
//     walked in chunks (whole groups of one colour) that all threads copy
//     into shared memory with coalesced 128-bit loads before processing;
//   * a thread owns one group (body pair) at a time and keeps the two
//     bodies' delta-v in registers across the group's contacts;
//   * every `check` sweeps the CTA evaluates the natural-map residual of its
//     scene and stops when it is below the target (or at the sweep cap);
//   * multipliers go back to the FP64 contact arrays and delta-v to the FP64
//     body arrays for integration.
// This is the FP32 path of the batched workload (the single-scene drop-in
// stays FP64).  CTA size and staging capacity are chosen by the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

static const int REC = 24;      // floats per packed contact record (global memory)
// a group's compact body id with GL_FIRST set: the group is the first, in
// colour order, to touch that body
static const int GL_FIRST = 1 << 30, GL_ID = GL_FIRST - 1;
static const int RECS = 28;     // shared-memory stride of a staged record: 7 float4 positions, see rec_pos
static const int MAXCB = 64;    // colours per scene
static const int MAXCH = 1024;  // staging chunks per scene

// Packed record (floats), 6 x 16 bytes:
//   [0..3]   n  and ra.x      [4..7]   t1 and ra.y      [8..11] t2 and ra.z
//   [12..15] rb and G21       [16..19] b0 b1 b2 G10     [20..23] 1/(D + c) of the rows, G20
// f = (n, t1, t2) is the contact frame, ra / rb the contact point from the
// two solve bodies' centres of mass.  The Jacobian rows are those of
// Contact.computeJacobian (Contact.java:199-255): (-f, f x ra, f, rb x f);
// the sweep forms them, and jinv J.w, from this and the bodies' inverse
// inertia, so a record is 96 bytes instead of the 256 of the full rows.
// Gqp = J_q M^-1 J_p^T are the couplings of the rows (with the sweep's own
// M^-1: minv and jinv of a pinned body count as 0).  The multipliers live in
// a separate array in the same slot order, 4 floats per slot: lambda of the
// three rows and the contact's friction coefficient mu (so a slot is one
// 16-byte copy); the multipliers are the only per-sweep writes.

__global__ void k_scene_ranges(const DPairs P, int npairs, const int* sceneOf, int nScenes, int* pairOff) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > npairs) return;
    int sp = p < npairs ? sceneOf[P.a[p]] : nScenes;
    int sq = p > 0 ? sceneOf[P.a[p - 1]] : -1;
    for (int s = sq + 1; s <= sp; s++) pairOff[s] = p;
}

__global__ void k_batch_pack(DBodies B, DContacts C, int nc, const int* slotOf, double comp, int fo, double fv,
                             float* rec, float* lamf) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int cap = C.cap;
    int sl = slotOf[c];
    float r[REC];
    for (int k = 0; k < REC; k++) r[k] = 0.f;
    const int ba = C.sb1[c], bb = C.sb2[c];
    for (int q = 0; q < 3; q++) {
        // f_q is the b.v part of row q
        for (int k = 0; k < 3; k++) r[4 * q + k] = (float)C.J[(12 * q + 6 + k) * cap + c];
        double D = C.bD[(3 + q) * cap + c];
        r[16 + q] = (float)C.bD[q * cap + c];
        r[20 + q] = (float)(1.0 / (D + comp));
        lamf[4 * sl + q] = (float)C.lam[q * cap + c];
    }
    // contact point (stored in body-1 coordinates) from both solve bodies
    {
        const int b1 = C.b1[c];
        v3 pB = mk(C.f[0 * cap + c], C.f[1 * cap + c], C.f[2 * cap + c]);
        v3 pW = add(mxv(ldm(B.R + 9 * b1), pB), ldv(B.x + 3 * b1));
        v3 ra = sub(pW, ldv(B.x + 3 * ba)), rb = sub(pW, ldv(B.x + 3 * bb));
        r[3] = (float)ra.x; r[7] = (float)ra.y; r[11] = (float)ra.z;
        r[12] = (float)rb.x; r[13] = (float)rb.y; r[14] = (float)rb.z;
    }
    // row couplings: the change of J_q . dv when row p moves by 1, through the
    // same delta-v update the sweep applies (linear parts scaled by minv,
    // angular parts by jinv J.w; both 0 for a pinned body)
    {
        double ma = (B.flags[ba] & F_PINNED) ? 0. : B.minv[ba];
        double mb = (B.flags[bb] & F_PINNED) ? 0. : B.minv[bb];
        auto G = [&](int q, int p) {
            double g = 0.;
            for (int k = 0; k < 3; k++) {
                g += ma * C.J[(12 * q + k) * cap + c] * C.J[(12 * p + k) * cap + c];
                g += C.J[(12 * q + 3 + k) * cap + c] * C.Ia[(3 * p + k) * cap + c];
                g += mb * C.J[(12 * q + 6 + k) * cap + c] * C.J[(12 * p + 6 + k) * cap + c];
                g += C.J[(12 * q + 9 + k) * cap + c] * C.Ib[(3 * p + k) * cap + c];
            }
            return (float)g;
        };
        r[19] = G(1, 0);
        r[23] = G(2, 0);
        r[15] = G(2, 1);
    }
    double mu;
    if (fo) mu = fv;
    else {
        double f1 = B.friction[C.b1[c]], f2 = B.friction[C.b2[c]];
        if (f1 < 0.2 || f2 < 0.2) mu = fmin(f1, f2);
        else if (f1 > 1. || f2 > 1.) mu = fmax(f1, f2);
        else mu = (f1 + f2) / 2.;
    }
    lamf[4 * sl + 3] = (float)mu;
    float4* dst = reinterpret_cast<float4*>(rec + (size_t)REC * sl);
    for (int k = 0; k < REC / 4; k++) dst[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
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
    const int CNTB = 16;                 // contact-count buckets for the order within a colour
    __shared__ int s_left, s_full, s_cnt[MAXCB + 1], s_bkt[MAXCB * CNTB];
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
    // Within a colour the groups are ordered by contact count, largest first:
    // a warp then takes groups of similar length, so its lanes idle less
    // while the longest group of the warp runs.  (Groups of one colour share
    // no body the sweep writes, so their order does not change results.)
    for (int k = t; k < MAXCB * CNTB; k += T) s_bkt[k] = 0;
    __syncthreads();
    auto bucket = [&](int g) { return CNTB - 1 - min(P.count[g], CNTB - 1); };
    for (int g = g0 + t; g < g1; g += T) {
        int c = colourOf[g];
        if (c >= 0) atomicAdd(&s_bkt[c * CNTB + bucket(g)], 1);
    }
    __syncthreads();
    if (t == 0) {
        if (s_left || s_full) dc->error = AM_E_CAPACITY;
        int ncol = 0;
        for (int k = 0; k < MAXCB; k++) if (s_cnt[k]) ncol = k + 1;
        int run = g0;
        for (int k = 0; k < ncol; k++) {
            colOff[s * (MAXCB + 1) + k] = run;
            for (int q = 0; q < CNTB; q++) { int n = s_bkt[k * CNTB + q]; s_bkt[k * CNTB + q] = run; run += n; }
        }
        for (int k = ncol; k <= MAXCB; k++) colOff[s * (MAXCB + 1) + k] = run;
    }
    __syncthreads();
    for (int g = g0 + t; g < g1; g += T) {
        int c = colourOf[g];
        if (c >= 0) gOrder[atomicAdd(&s_bkt[c * CNTB + bucket(g)], 1)] = g;
    }
}

__device__ __forceinline__ int scene_colours(const int* co) {
    int n = 0;
    while (n < MAXCB && co[n + 1] > co[n]) n++;
    return n;
}

// Slots of one scene (one CTA per scene): the groups in colour order get
// consecutive slot runs (an exclusive scan of their contact counts); the
// scene is cut into chunks of whole groups of one colour whose records fit
// `cap` slots.  A chunk head entry carries bit 30 when it starts a colour.
__global__ void k_batch_slots(DContacts C, DPairs P, const int* pairOff, const int* gOrder, const int* colOff,
                              const int* sceneBodyOff, int nc, int npairs, int cap, int2* gInfo, int2* glid,
                              int* slotOf, int* contactOf, int* chunkK, int* nChunks, int2* sceneSize,
                              int* lidOf, int* bodyOf, int* sceneActive, DCount* dc) {
    extern __shared__ int s_lid[];   // [bodies of the scene]: active flag, then compact id (-1: inactive)
    __shared__ int s_carry, s_maxcnt, s_warp[32], s_colch[MAXCB + 1];
    const unsigned FULL = 0xffffffffu;
    int s = blockIdx.x, t = threadIdx.x, T = blockDim.x;
    int lane = t & 31, w = t >> 5, nw = T >> 5;
    int g0 = pairOff[s];
    const int* co = colOff + s * (MAXCB + 1);
    int ncol = scene_colours(co);
    int kEnd = co[ncol];
    int slot0 = g0 < npairs ? P.off[g0] : nc;
    int b0 = sceneBodyOff[s];
    if (t == 0) { s_carry = 0; s_maxcnt = 0; }
    __syncthreads();
    for (int base = g0; base < kEnd; base += T) {
        int k = base + t;
        int cnt = 0, g = 0;
        if (k < kEnd) { g = gOrder[k]; cnt = P.count[g]; }
        int x = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[w] = x;
        __syncthreads();
        if (w == 0) {
            int v = lane < nw ? s_warp[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(FULL, v, o);
                if (lane >= o) v += y;
            }
            if (lane < nw) s_warp[lane] = v;
        }
        __syncthreads();
        int excl = s_carry + (w ? s_warp[w - 1] : 0) + x - cnt;
        if (k < kEnd) {
            int sl = slot0 + excl;
            int c0 = P.off[g];
            gInfo[k] = make_int2(sl, cnt);
            glid[k] = make_int2(C.sb1[c0] - b0, C.sb2[c0] - b0);
            for (int j = 0; j < cnt; j++) { slotOf[c0 + j] = sl + j; contactOf[sl + j] = c0 + j; }
            atomicMax(&s_maxcnt, cnt);
        }
        __syncthreads();
        if (t == 0) s_carry += s_warp[nw - 1];
        __syncthreads();
    }
    const int maxc = s_maxcnt, nslots = s_carry;
    // Active bodies (those in some group of the scene) get compact ids in
    // body order: the sweep keeps delta-v, inverse mass and inertia only for
    // them, and a body without contacts gets delta-v 0.
    {
        const int nb = sceneBodyOff[s + 1] - b0;
        for (int b = t; b < nb; b += T) s_lid[b] = 0;
        __syncthreads();
        for (int k = g0 + t; k < kEnd; k += T) {
            int2 l = glid[k];
            s_lid[l.x] = 1;
            s_lid[l.y] = 1;
        }
        __syncthreads();
        if (t == 0) s_carry = 0;
        __syncthreads();
        for (int base = 0; base < nb; base += T) {
            int b = base + t;
            int f = b < nb ? s_lid[b] : 0;
            int x = f;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(FULL, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) s_warp[w] = x;
            __syncthreads();
            if (w == 0) {
                int v = lane < nw ? s_warp[lane] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    int y = __shfl_up_sync(FULL, v, o);
                    if (lane >= o) v += y;
                }
                if (lane < nw) s_warp[lane] = v;
            }
            __syncthreads();
            int id = s_carry + (w ? s_warp[w - 1] : 0) + x - f;
            if (b < nb) {
                s_lid[b] = f ? id : -1;
                lidOf[b0 + b] = f ? id : -1;
                if (f) bodyOf[b0 + id] = b0 + b;
            }
            __syncthreads();
            if (t == 0) s_carry += s_warp[nw - 1];
            __syncthreads();
        }
        if (t == 0) sceneActive[s] = s_carry;
        for (int k = g0 + t; k < kEnd; k += T) {
            int2 l = glid[k];
            glid[k] = make_int2(s_lid[l.x], s_lid[l.y]);
        }
        __syncthreads();
        // the first group (in colour order) that touches each active body
        // carries GL_FIRST on that body's id: a sweep that walks the colours
        // in order reaches the body there first
        const int nbA = s_carry;
        for (int b = t; b < nbA; b += T) s_lid[b] = 0x7FFFFFFF;
        __syncthreads();
        for (int k = g0 + t; k < kEnd; k += T) {
            int2 l = glid[k];
            atomicMin(&s_lid[l.x], k);
            atomicMin(&s_lid[l.y], k);
        }
        __syncthreads();
        for (int k = g0 + t; k < kEnd; k += T) {
            int2 l = glid[k];
            glid[k] = make_int2(l.x | (s_lid[l.x] == k ? GL_FIRST : 0), l.y | (s_lid[l.y] == k ? GL_FIRST : 0));
        }
        __syncthreads();
    }
    // slots of the scene, and the most a split of every colour into equal
    // slot windows can add to one part: one group per colour, plus one slot
    // per colour for rounding the window bounds
    if (t == 0) sceneSize[s] = make_int2(nslots, ncol * (maxc + 1));
    int win = cap - maxc;
    if (win < maxc || win <= 0) {   // a group larger than half the staging buffer
        if (t == 0) { dc->error = AM_E_CAPACITY; nChunks[s] = 0; }
        return;
    }
    for (int col = t; col < ncol; col += T) {
        int st = gInfo[co[col]].x;
        s_colch[col] = (gInfo[co[col + 1] - 1].x - st) / win + 1;
    }
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int col = 0; col < ncol; col++) { int n = s_colch[col]; s_colch[col] = run; run += n; }
        s_colch[ncol] = run;
        if (run > MAXCH) { dc->error = AM_E_CAPACITY; run = 0; }
        nChunks[s] = run;
        chunkK[s * (MAXCH + 1) + run] = kEnd | (1 << 30);
    }
    __syncthreads();
    if (s_colch[ncol] > MAXCH) return;
    for (int k = g0 + t; k < kEnd; k += T) {
        int col = 0;
        while (co[col + 1] <= k) col++;
        int st = gInfo[co[col]].x;
        int j = (gInfo[k].x - st) / win;
        bool chead = k == co[col];
        if (chead || (gInfo[k - 1].x - st) / win != j)
            chunkK[s * (MAXCH + 1) + s_colch[col] + j] = k | (chead ? (1 << 30) : 0);
    }
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 sld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ long long gtimer() {
    long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    return v;
}
__device__ __forceinline__ int smid() {
    int v;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(v));
    return v;
}
// world inverse inertia of a body as its symmetric part (xx yy zz xy xz yz),
// 0 for a pinned body
__device__ __forceinline__ void load_jinv(const DBodies& B, int b, bool pinned, float* o) {
    const double* J = B.jinv + 9 * (size_t)b;
    const int idx[6] = {0, 4, 8, 1, 2, 5};
    for (int k = 0; k < 6; k++) o[k] = pinned ? 0.f : (float)J[idx[k]];
}
// solve start and end of a scene and the SM that ran it
__device__ __forceinline__ void trace_scene(long long* trace, int s, long long t0) {
    if (!trace) return;
    trace[3 * s] = t0;
    trace[3 * s + 1] = gtimer();
    trace[3 * s + 2] = smid();
}

// A body pair's state across one group: both bodies' delta-v (v, w), world
// inverse inertia (symmetric: xx yy zz xy xz yz) and inverse mass (0 for a
// pinned body, whose delta-v is never written back).
struct Pair {
    float a[6], b[6];
    float ja[6], jb[6];
    float ma, mb;
};

// One contact record in registers (layout above).
struct Rec {
    float f[3][3];      // n, t1, t2
    float ra[3], rb[3]; // contact point from each body's centre of mass
    float bq[3], iq[3]; // b and 1 / (D + c) of the three rows
    float g10, g20, g21;
};

// Position (in float4 units) of 16-byte piece q of the record staged at
// shared-memory slot `slot`: the pieces rotate by (slot / 8) mod 7 through the
// slot's 7 positions.  Threads of a warp read the same piece of records whose
// slots differ by a group's contact count; without the rotation the pieces of
// groups with 4 or 8 contacts fall on the same shared-memory banks.
__device__ __forceinline__ int rec_rot(int slot) { return (slot >> 3) % 7; }
__device__ __forceinline__ int rec_pos(int rot, int q) { int p = q + rot; return p >= 7 ? p - 7 : p; }

// Shared-memory slot of the multipliers of staged slot `slot`: the low three
// bits are XORed with the next three (a permutation within each aligned run
// of 8 slots), so the groups of one warp, whose slots differ by their contact
// count, read and write different banks.
__device__ __forceinline__ int lam_pos(int slot) { return slot ^ ((slot >> 3) & 7); }

__device__ __forceinline__ void load_rec(const float* R, int slot, Rec& c) {
    const int rot = rec_rot(slot);
    const float4 q0 = sld4(R + 4 * rec_pos(rot, 0)), q1 = sld4(R + 4 * rec_pos(rot, 1)),
                 q2 = sld4(R + 4 * rec_pos(rot, 2)), q3 = sld4(R + 4 * rec_pos(rot, 3)),
                 q4 = sld4(R + 4 * rec_pos(rot, 4)), q5 = sld4(R + 4 * rec_pos(rot, 5));
    c.f[0][0] = q0.x; c.f[0][1] = q0.y; c.f[0][2] = q0.z; c.ra[0] = q0.w;
    c.f[1][0] = q1.x; c.f[1][1] = q1.y; c.f[1][2] = q1.z; c.ra[1] = q1.w;
    c.f[2][0] = q2.x; c.f[2][1] = q2.y; c.f[2][2] = q2.z; c.ra[2] = q2.w;
    c.rb[0] = q3.x; c.rb[1] = q3.y; c.rb[2] = q3.z; c.g21 = q3.w;
    c.bq[0] = q4.x; c.bq[1] = q4.y; c.bq[2] = q4.z; c.g10 = q4.w;
    c.iq[0] = q5.x; c.iq[1] = q5.y; c.iq[2] = q5.z; c.g20 = q5.w;
}

// w x r
__device__ __forceinline__ void cross3(const float* w, const float* r, float* o) {
    o[0] = fmaf(w[1], r[2], -w[2] * r[1]);
    o[1] = fmaf(w[2], r[0], -w[0] * r[2]);
    o[2] = fmaf(w[0], r[1], -w[1] * r[0]);
}
// o += symmetric matrix (xx yy zz xy xz yz) times v, accumulated inside the
// FMA chain
__device__ __forceinline__ void symv_acc(const float* m, const float* v, float* o) {
    o[0] = fmaf(m[4], v[2], fmaf(m[3], v[1], fmaf(m[0], v[0], o[0])));
    o[1] = fmaf(m[5], v[2], fmaf(m[1], v[1], fmaf(m[3], v[0], o[1])));
    o[2] = fmaf(m[2], v[2], fmaf(m[5], v[1], fmaf(m[4], v[0], o[2])));
}

// Velocity of the contact point on body b relative to body a:
// J_q . dv = f_q . rv for the Jacobian rows of Contact.computeJacobian
// (-f, f x ra, f, rb x f).
__device__ __forceinline__ void rel_vel(const Pair& P, const Rec& c, float* rv) {
    float wa[3], wb[3];
    cross3(P.a + 3, c.ra, wa);
    cross3(P.b + 3, c.rb, wb);
    for (int k = 0; k < 3; k++) rv[k] = (P.b[k] - P.a[k]) + (wb[k] - wa[k]);
}
__device__ __forceinline__ float fdot(const float* f, const float* v) {
    return fmaf(f[2], v[2], fmaf(f[1], v[1], f[0] * v[0]));
}

// delta-v += M^-1 J^T for the impulse F (world frame, the sum of d_q f_q of
// the rows): linear parts -ma F and mb F, angular jinv (F x ra), jinv (rb x F)
__device__ __forceinline__ void pair_impulse(Pair& P, const Rec& c, const float* F) {
    float u[3], w[3];
    cross3(F, c.ra, u);
    cross3(c.rb, F, w);
    symv_acc(P.ja, u, P.a + 3);
    symv_acc(P.jb, w, P.b + 3);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        P.a[k] = fmaf(-P.ma, F[k], P.a[k]);
        P.b[k] = fmaf(P.mb, F[k], P.b[k]);
    }
}

// One contact of a Gauss-Seidel sweep (PGS.java:120-160): the normal row,
// then the two friction rows boxed by mu times the new normal multiplier.
// All three rows take J . dv at the contact's start state, and the friction
// rows add what the earlier rows of the same contact changed, through the
// couplings G10, G20, G21 of the record.  In exact arithmetic this is the
// row-by-row update; the dependent chain is one relative velocity, three
// scalar updates and one impulse (the three rows' changes applied together)
// instead of three dot products and three updates.  (D lam - w) / (D + c) is
// evaluated as lam - (c lam + w) / (D + c), and the relaxation factor (1:
// plain) scales 1 / (D + c).
__device__ __forceinline__ void sweep_contact_l(Pair& P, const float* R, int slot, const float4 l, float* lp,
                                                float omega, float comp, float relax, float* dOut) {
    Rec c;
    load_rec(R, slot, c);
    float rv[3];
    rel_vel(P, c, rv);
    const float lq[3] = {l.x, l.y, l.z};
    // row q unclamped: lam_q + ni_q (k_q + omega (p_q + sum_p G_qp d_p)), with
    // ni = -relax / (D + c) and k = c lam + omega b; the base at the start state
    // and the coupling factors are formed off the dependent chain
    float base[3], ni[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        ni[q] = -relax * c.iq[q];
        const float k = fmaf(comp, lq[q], omega * c.bq[q]);
        base[q] = fmaf(ni[q], fmaf(omega, fdot(c.f[q], rv), k), lq[q]);
    }
    const float c10 = ni[1] * omega * c.g10, c20 = ni[2] * omega * c.g20, c21 = ni[2] * omega * c.g21;
    const float n0 = fmaxf(base[0], 0.f);
    const float d0 = n0 - l.x;
    const float lim = l.w * n0;   // mu n0
    const float n1 = fminf(fmaxf(fmaf(c10, d0, base[1]), -lim), lim);
    const float d1 = n1 - l.y;
    const float n2 = fminf(fmaxf(fmaf(c21, d1, fmaf(c20, d0, base[2])), -lim), lim);
    const float d2 = n2 - l.z;
    dOut[0] = d0;
    dOut[1] = d1;
    dOut[2] = d2;
    *reinterpret_cast<float4*>(lp) = make_float4(n0, n1, n2, l.w);
    float F[3];
#pragma unroll
    for (int q = 0; q < 3; q++) F[q] = fmaf(d2, c.f[2][q], fmaf(d1, c.f[1][q], d0 * c.f[0][q]));
    pair_impulse(P, c, F);
}

__device__ __forceinline__ void sweep_contact(Pair& P, const float* R, int slot, float* lp, float omega,
                                              float comp, float relax, float* dOut) {
    sweep_contact_l(P, R, slot, sld4(lp), lp, omega, comp, relax, dOut);
}

// PGS.confidentWarmStart: delta-v += M^-1 J^T lambda
__device__ __forceinline__ void warm_contact(Pair& P, const float* R, int slot, const float* lp) {
    Rec c;
    load_rec(R, slot, c);
    const float4 l = sld4(lp);
    float F[3];
#pragma unroll
    for (int q = 0; q < 3; q++) F[q] = fmaf(l.z, c.f[2][q], fmaf(l.y, c.f[1][q], l.x * c.f[0][q]));
    pair_impulse(P, c, F);
}

// natural-map residual of a contact at the current state:
// |lambda - proj(lambda - (b + J dv + c lambda) / (D + c))|
__device__ __forceinline__ void res_contact(const Pair& P, const float* R, int slot, const float* lp, float comp,
                                            float& rmax,
                                            float& lmax) {
    Rec c;
    load_rec(R, slot, c);
    const float4 l = sld4(lp);
    const float lq[3] = {l.x, l.y, l.z};
    float rv[3];
    rel_vel(P, c, rv);
    // explicit roundings: every kernel that inlines this evaluates the same
    // operations, so a scene stops at the same check whichever kernel solves it
#pragma unroll
    for (int q = 0; q < 3; q++) {
        float w = __fmaf_rn(comp, lq[q], __fadd_rn(c.bq[q], fdot(c.f[q], rv)));
        float z = __fmaf_rn(-w, c.iq[q], lq[q]);
        if (q == 0) z = fmaxf(z, 0.f);
        else { float lim = l.w * l.x; z = fminf(fmaxf(z, -lim), lim); }
        rmax = fmaxf(rmax, fabsf(lq[q] - z));
        lmax = fmaxf(lmax, fabsf(lq[q]));
    }
}

// Contact.updateContactState after the final sweep: broken when the normal
// multiplier vanished, on edge when a tangential velocity exceeds `slide`
__device__ __forceinline__ int final_state(const Pair& P, const float* R, int slot, const float* lp, float slide) {
    Rec c;
    load_rec(R, slot, c);
    float rv[3];
    rel_vel(P, c, rv);
    const float w1 = __fadd_rn(c.bq[1], fdot(c.f[1], rv)), w2 = __fadd_rn(c.bq[2], fdot(c.f[2], rv));
    if (fabsf(lp[0]) <= 1e-14f) return AM_STATE_BROKEN;
    if (fabsf(w1) > slide || fabsf(w2) > slide) return AM_STATE_ONEDGE;
    return AM_STATE_CLEAR;
}

// ---------------------------------------------------------------------------
// Nonsmooth nonlinear conjugate gradient (NNCG; Silcowitz, Niebe and Erleben,
// 2010) around the projected Gauss-Seidel sweep.  With g the change of the
// multipliers over one sweep and beta = |g_k|^2 / |g_k-1|^2: beta > 1
// restarts (p = 0); otherwise lambda += beta p and p = beta p + g.  The
// fixed point is that of PGS, so the residual stopping rule is unchanged.
// The momentum's effect on delta-v, beta M^-1 J^T p, is kept per body as
// q = M^-1 J^T p, which follows q = beta q + (the sweep's own delta-v
// change); the momentum step is then one pass over slots and one over bodies,
// with no colour order.
//
// |g|^2 must come out bit-identical whatever CTA size, size class, staging
// or cluster solves the scene, and whatever order the groups of a colour
// take (the colouring places them by atomic arrival).  So it is summed
// exactly, in integers: each group's squared change (a float, summed over
// its contacts in slot order) is scaled by 2^E and rounded to a 64-bit
// integer, and integer sums do not depend on their order.  Four scales
// E0 + 16j run side by side (E0 from the previous sweep's |g|^2, or a fixed
// one on the first sweep); the finest whose total stays below 2^50 (so no
// group was clamped) gives |g|^2.
static const int NNCG_SCALES = 4;
static const unsigned long long NNCG_CLAMP = 1ull << 50;

// E0 of the sweep after one whose |g|^2 was gg (the first sweep: -10)
__device__ __forceinline__ int nncg_e0(int it, float gg) {
    if (it == 0) return -10;
    const float x = fminf(fmaxf(gg, 0x1p-100f), 0x1p100f);
    return 10 - (((int)(__float_as_uint(x) >> 23) & 255) - 127);   // 10 - floor(log2 x)
}
// x * 2^E rounded (half up) to an integer, clamped to 2^50; x >= 0 and
// finite (zero and subnormal x lie below every scale used)
__device__ __forceinline__ unsigned long long nncg_fixed(float x, int E) {
    const unsigned b = __float_as_uint(x);
    const int e = (int)(b >> 23) & 255;
    if (e == 0) return 0ull;
    const unsigned long long m = (b & 0x7FFFFFu) | 0x800000u;   // x = m 2^(e - 150)
    const int sh = e - 150 + E;
    if (sh >= 27) return NNCG_CLAMP;                               // m 2^sh >= 2^50
    if (sh >= 0) return min(m << sh, NNCG_CLAMP);
    if (sh < -25) return 0ull;
    return (m + (1ull << (-sh - 1))) >> (-sh);
}
// a thread's |g|^2 accumulators at the four scales (named fields, so they
// stay in registers inside the kernels' lambdas)
struct Acc4 {
    unsigned long long a0 = 0ull, a1 = 0ull, a2 = 0ull, a3 = 0ull;
};
// one group's squared change at the four scales, added to acc
__device__ __forceinline__ void nncg_acc(float gsq, int e0, Acc4& acc) {
    acc.a0 += nncg_fixed(gsq, e0);
    acc.a1 += nncg_fixed(gsq, e0 + 16);
    acc.a2 += nncg_fixed(gsq, e0 + 32);
    acc.a3 += nncg_fixed(gsq, e0 + 48);
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// a warp's accumulators into the CTA's shared totals (integer: any order)
__device__ __forceinline__ void nncg_flush(Acc4& acc, unsigned long long* tot) {
    const unsigned long long v0 = warp_sum_u64(acc.a0), v1 = warp_sum_u64(acc.a1), v2 = warp_sum_u64(acc.a2),
                             v3 = warp_sum_u64(acc.a3);
    if ((threadIdx.x & 31) == 0) {
        if (v0) atomicAdd(tot + 0, v0);
        if (v1) atomicAdd(tot + 1, v1);
        if (v2) atomicAdd(tot + 2, v2);
        if (v3) atomicAdd(tot + 3, v3);
    }
    acc = Acc4();
}
// |g|^2 from the totals of the four scales
__device__ __forceinline__ float nncg_gg(const unsigned long long* tot, int e0) {
    // the finest scale below the clamp (no dynamic index: tot may be registers)
    const unsigned long long t0 = tot[0], t1 = tot[1], t2 = tot[2], t3 = tot[3];
    const int j = t3 < NNCG_CLAMP ? 3 : (t2 < NNCG_CLAMP ? 2 : (t1 < NNCG_CLAMP ? 1 : 0));
    const unsigned long long tj = j == 3 ? t3 : (j == 2 ? t2 : (j == 1 ? t1 : t0));
    // the power-of-two scale 2^-E is applied in two exact steps, each a float
    // built from its exponent bits
    const int E = e0 + 16 * j;
    const int h1 = -E / 2, h2 = -E - h1;   // both within the normal exponent range
    return __fmul_rn(__fmul_rn(__ull2float_rn(tj), __int_as_float((h1 + 127) << 23)),
                     __int_as_float((h2 + 127) << 23));
}
// the sweep's squared change of one contact, accumulated in a fixed order
__device__ __forceinline__ float sq3_acc(const float* d, float acc) {
    return __fmaf_rn(d[2], d[2], __fmaf_rn(d[1], d[1], __fmaf_rn(d[0], d[0], acc)));
}
// beta of iteration `it` (0: the first sweep, no momentum); < 0 means restart
__device__ __forceinline__ float nncg_beta(int it, float gg, float ggPrev) {
    if (it == 0) return 0.f;
    const float b = __fdiv_rn(gg, ggPrev);
    return (b <= 1.f) ? b : -1.f;   // also restarts on 0 / 0 and overflow
}
// one slot: lambda (xyz of the 16-byte multiplier slot, w = mu), g and p
// (gp[0..2] and gp[4..6]; both 16-byte aligned, read and written as float4
// so the 32-byte stride between slots costs few shared-memory wavefronts)
__device__ __forceinline__ void nncg_slot(float* l, float* gp, int it, float beta) {
    float4 L = *reinterpret_cast<float4*>(l);
    const float4 g = *reinterpret_cast<const float4*>(gp);
    float4 p = *reinterpret_cast<const float4*>(gp + 4);
    if (it == 0) {
        p = g;
    } else if (beta < 0.f) {
        p = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        L.x = __fmaf_rn(beta, p.x, L.x);
        L.y = __fmaf_rn(beta, p.y, L.y);
        L.z = __fmaf_rn(beta, p.z, L.z);
        p = make_float4(__fmaf_rn(beta, p.x, g.x), __fmaf_rn(beta, p.y, g.y), __fmaf_rn(beta, p.z, g.z), 0.f);
        *reinterpret_cast<float4*>(l) = L;
    }
    *reinterpret_cast<float4*>(gp + 4) = p;
}
// nncg_slot on a multiplier slot already in registers (the sweep update that
// follows loads and stores it once)
__device__ __forceinline__ float4 nncg_slot_reg(float4 L, float* gp, int it, float beta) {
    const float4 g = *reinterpret_cast<const float4*>(gp);
    float4 p = *reinterpret_cast<const float4*>(gp + 4);
    if (it == 0) {
        p = g;
    } else if (beta < 0.f) {
        p = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        L.x = __fmaf_rn(beta, p.x, L.x);
        L.y = __fmaf_rn(beta, p.y, L.y);
        L.z = __fmaf_rn(beta, p.z, L.z);
        p = make_float4(__fmaf_rn(beta, p.x, g.x), __fmaf_rn(beta, p.y, g.y), __fmaf_rn(beta, p.z, g.z), 0.f);
    }
    *reinterpret_cast<float4*>(gp + 4) = p;
    return L;
}
// one body's momentum step on delta-v v, delta-v at the sweep's start d0 and
// q (6 each): q = beta q + (v - d0), v += beta q_old, d0 = v (first
// iteration: q = v - d0; restart: q = 0)
__device__ __forceinline__ void nncg_body_core(float* v, float* d0, float* q, int it, float beta) {
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const float d = __fsub_rn(v[k], d0[k]);
        if (it == 0) {
            q[k] = d;
        } else if (beta < 0.f) {
            q[k] = 0.f;
        } else {
            v[k] = __fmaf_rn(beta, q[k], v[k]);
            q[k] = __fmaf_rn(beta, q[k], d);
        }
        d0[k] = v[k];
    }
}
// dq (12 floats, 16-byte aligned): delta-v at the sweep's start, then q
__device__ __forceinline__ void dq_unpack(float4 a, float4 b, float4 c, float* d0, float* q) {
    d0[0] = a.x; d0[1] = a.y; d0[2] = a.z; d0[3] = a.w;
    d0[4] = b.x; d0[5] = b.y; q[0] = b.z; q[1] = b.w;
    q[2] = c.x; q[3] = c.y; q[4] = c.z; q[5] = c.w;
}
// one body in memory: delta-v (6 floats, 8-byte aligned) and dq
__device__ __forceinline__ void nncg_body(float* dv, float* dq, int it, float beta) {
    float v[6], d0[6], q[6];
    const float2* v2 = reinterpret_cast<const float2*>(dv);
    const float4* q4 = reinterpret_cast<const float4*>(dq);
#pragma unroll
    for (int k = 0; k < 3; k++) { const float2 a = v2[k]; v[2 * k] = a.x; v[2 * k + 1] = a.y; }
    dq_unpack(q4[0], q4[1], q4[2], d0, q);
    nncg_body_core(v, d0, q, it, beta);
    float2* w2 = reinterpret_cast<float2*>(dv);
    float4* w4 = reinterpret_cast<float4*>(dq);
#pragma unroll
    for (int k = 0; k < 3; k++) w2[k] = make_float2(v[2 * k], v[2 * k + 1]);
    w4[0] = make_float4(d0[0], d0[1], d0[2], d0[3]);
    w4[1] = make_float4(d0[4], d0[5], q[0], q[1]);
    w4[2] = make_float4(q[2], q[3], q[4], q[5]);
}
// the same step on a body whose delta-v is in registers (a group's first
// touch of the body in a sweep) and whose dq is in this CTA's shared memory
// or in global memory
__device__ __forceinline__ void nncg_body_reg(float* v, float* dq, int it, float beta) {
    float d0[6], q[6];
    const float4* q4 = reinterpret_cast<const float4*>(dq);
    dq_unpack(q4[0], q4[1], q4[2], d0, q);
    nncg_body_core(v, d0, q, it, beta);
    float4* w4 = reinterpret_cast<float4*>(dq);
    w4[0] = make_float4(d0[0], d0[1], d0[2], d0[3]);
    w4[1] = make_float4(d0[4], d0[5], q[0], q[1]);
    w4[2] = make_float4(q[2], q[3], q[4], q[5]);
}

// shared-memory layout of the sweep kernel (floats).  The staging arrays
// hold two buffers of `cap` slots each (double buffering of chunks); a
// resident scene uses both as one buffer of 2 cap slots.
// With the conjugate-gradient acceleration on, a resident scene also keeps
// per body delta-v at the sweep's start and q (12 floats) and per slot g and
// p (8 floats, at the multipliers' permuted position); a streamed scene keeps
// these in global memory.
struct SweepSmem {
    int dv, mv, ji, dq, rec, lam, gp, gi, gl, total;
    __host__ __device__ SweepSmem(int nbMax, int cap, int accel = 0) {
        dv = 0;                // 6 floats per body (even offsets: 8-byte aligned)
        ji = 6 * nbMax;        // symmetric inverse inertia, 6 floats per body
        dq = 12 * nbMax;       // accel: delta-v at sweep start and q, 12 floats per body
        mv = dq + (accel ? 12 * nbMax : 0);
        rec = (mv + nbMax + 3) & ~3;
        lam = rec + 2 * cap * RECS;
        gp = lam + 8 * cap;
        gi = gp + (accel ? 16 * cap : 0);
        gl = gi + 4 * cap;
        total = gl + 4 * cap;
    }
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

enum { OP_WARM = 0, OP_SWEEP = 1, OP_RES = 2, OP_FINAL = 3 };

__global__ void __launch_bounds__(512) k_batch_sweep(
    DBodies B, DContacts C, const int* sceneBodyOff, const int* sceneOrder, const int2* gInfo, const int2* glid,
    const int* chunkK, const int* nChunks, const int* contactOf, const float* __restrict__ rec, float* lamS, int cap,
    int nbMax, int iters, float omega, float comp, float tolRel, int check, float slide, int* sceneSweeps,
    float* sceneRes, const float* lamAlt, int* sceneFall, int writeBack, int inner, float relax, int sym,
    long long* trace, const int* lidOf, const int* bodyOf, const int* sceneActive, int accel, float* gpG,
    float* dqG) {
    extern __shared__ float sm[];
    const SweepSmem L(nbMax, cap, accel);
    const long long tStart = gtimer();
    float* dv = sm + L.dv;
    float* mv = sm + L.mv;
    float* ji = sm + L.ji;
    float* srec = sm + L.rec;
    float* slam = sm + L.lam;
    int2* sgi = reinterpret_cast<int2*>(sm + L.gi);
    int2* sgl = reinterpret_cast<int2*>(sm + L.gl);
    __shared__ float s_res, s_lam;
    __shared__ int s_stop;
    const int s = sceneOrder ? sceneOrder[blockIdx.x] : blockIdx.x;
    const int t = threadIdx.x, T = blockDim.x;
    const int b0 = sceneBodyOff[s], nb = sceneBodyOff[s + 1] - b0;
    const int* ck = chunkK + s * (MAXCH + 1);
    const int nch = nChunks[s];
    const int HEAD = 1 << 30, KMASK = HEAD - 1;
    // a scene without contacts touches no shared memory (its launch may lay
    // out none for its bodies)
    if (nch == 0) {
        if (!writeBack) return;
        for (int b = t; b < nb; b += T)
            for (int k = 0; k < 6; k++) B.dv[6 * (b0 + b) + k] = 0.0;
        if (t == 0) {
            sceneSweeps[s] = 0;
            sceneRes[s] = 0.f;
            if (sceneFall) sceneFall[s] = 0;
            trace_scene(trace, s, tStart);
        }
        return;
    }
    // the scene's active bodies (compact ids).  Pinned bodies get 0 here, the
    // same test the colouring uses to let groups of one colour share them;
    // their delta-v is never written
    const int nbA = sceneActive[s];
    for (int b = t; b < nbA; b += T) {
        const int gb = bodyOf[b0 + b];
        const bool pin = (B.flags[gb] & F_PINNED) != 0;
        mv[b] = pin ? 0.f : (float)B.minv[gb];
        for (int k = 0; k < 6; k++) dv[6 * b + k] = 0.f;
        load_jinv(B, gb, pin, ji + 6 * b);
    }
    const int kS0 = ck[0] & KMASK, kS1 = ck[nch] & KMASK;
    const int slotS0 = gInfo[kS0].x;
    const int2 lastG = gInfo[kS1 - 1];
    const int nslots = lastG.x + lastG.y - slotS0;
    const bool resident = nslots <= 2 * cap;
    // conjugate-gradient state: shared memory for a resident scene, global
    // memory (slot and body arrays of the whole batch) for a streamed one;
    // |g|^2 totals by sweep parity
    __shared__ unsigned long long s_tot[2][NNCG_SCALES];
    float* sgp = sm + L.gp;
    float* dqB = resident ? sm + L.dq : dqG + 12 * (size_t)b0;
    Acc4 acc;
    int e0 = 0, par = 0;

    // issue the asynchronous copy of groups [k0, k1) (and their slots) into
    // staging buffer `buf` (one commit group per call)
    auto stage = [&](int buf, int k0, int k1) {
        int s0 = gInfo[k0].x;
        int2 e = gInfo[k1 - 1];
        int nsl = e.x + e.y - s0;
        for (int i = t; i < nsl * (REC / 4); i += T) {
            int sl = i / (REC / 4), q = i - sl * (REC / 4);
            int bs = buf * cap + sl;   // slot in the staging buffers
            cp_async16(srec + bs * RECS + 4 * rec_pos(rec_rot(bs), q), rec + (size_t)(s0 + sl) * REC + 4 * q);
        }
        for (int i = t; i < nsl; i += T) cp_async16(slam + 4 * lam_pos(buf * cap + i), lamS + 4 * ((size_t)s0 + i));
        for (int i = t; i < k1 - k0; i += T) {
            cp_async8(sgi + buf * cap + i, gInfo + k0 + i);
            cp_async8(sgl + buf * cap + i, glid + k0 + i);
        }
        cp_async_commit();
    };
    // multipliers of a staged chunk back to global memory
    auto unstage = [&](int buf, int k0, int k1) {
        int s0 = gInfo[k0].x;
        int2 e = gInfo[k1 - 1];
        int nsl = e.x + e.y - s0;
        for (int i = t; i < nsl; i += T)
            *reinterpret_cast<float4*>(lamS + 4 * ((size_t)s0 + i)) =
                *reinterpret_cast<const float4*>(slam + 4 * lam_pos(buf * cap + i));
    };

    float rmax = 0.f, lmax = 0.f;
    // one group: its two bodies' delta-v in registers across its contacts;
    // sl0 is the group's first slot in the staging buffer, slA in the scene
    // a momentum step left pending by the previous sweep (pendIt, pendBeta):
    // applied to each body at its first touch and to each slot before its
    // update, the same arithmetic as the eager passes
    bool pend = false;
    int pendIt = 0;
    float pendBeta = 0.f;
    auto group = [&](int op, int sl0, int slA, int cnt, int2 idf) {
        const int2 id = make_int2(idf.x & GL_ID, idf.y & GL_ID);
        Pair P;
        {   // 8-byte aligned: 6 floats per body from an even offset
            const float2* da = reinterpret_cast<const float2*>(dv + 6 * id.x);
            const float2* db = reinterpret_cast<const float2*>(dv + 6 * id.y);
            const float2* ja = reinterpret_cast<const float2*>(ji + 6 * id.x);
            const float2* jb = reinterpret_cast<const float2*>(ji + 6 * id.y);
            for (int q = 0; q < 3; q++) {
                float2 u = da[q], v = db[q], x = ja[q], y = jb[q];
                P.a[2 * q] = u.x; P.a[2 * q + 1] = u.y;
                P.b[2 * q] = v.x; P.b[2 * q + 1] = v.y;
                P.ja[2 * q] = x.x; P.ja[2 * q + 1] = x.y;
                P.jb[2 * q] = y.x; P.jb[2 * q + 1] = y.y;
            }
        }
        P.ma = mv[id.x];
        P.mb = mv[id.y];
        const bool lazy = op == OP_SWEEP && pend;
        if (lazy) {
            if ((idf.x & GL_FIRST) && P.ma != 0.f) nncg_body_reg(P.a, dqB + 12 * id.x, pendIt, pendBeta);
            if ((idf.y & GL_FIRST) && P.mb != 0.f) nncg_body_reg(P.b, dqB + 12 * id.y, pendIt, pendBeta);
        }
        // sweeps may pass over a group's contacts `inner` times: Gauss-Seidel
        // on the body pair's own block before the sweep moves on
        const int reps = op == OP_SWEEP ? inner : 1;
        float gsq = 0.f;
        for (int rep = 0; rep < reps; rep++)
        for (int j = 0; j < cnt; j++) {
            const int slot = sl0 + j;
            const float* R = srec + slot * RECS;
            float* lp = slam + 4 * lam_pos(slot);
            if (op == OP_WARM) {
                warm_contact(P, R, slot, lp);
            } else if (op == OP_SWEEP) {
                float d[3];
                float* g = accel ? (resident ? sgp + 8 * lam_pos(slot) : gpG + 8 * ((size_t)slA + j)) : nullptr;
                float4 l = sld4(lp);
                if (lazy && rep == 0) l = nncg_slot_reg(l, g, pendIt, pendBeta);
                sweep_contact_l(P, R, slot, l, lp, omega, comp, relax, d);
                if (accel) {
                    if (rep > 0)
                        for (int q = 0; q < 3; q++) d[q] = __fadd_rn(g[q], d[q]);
                    *reinterpret_cast<float4*>(g) = make_float4(d[0], d[1], d[2], 0.f);
                    if (rep == reps - 1) gsq = sq3_acc(d, gsq);
                }
            } else if (op == OP_RES) {
                res_contact(P, R, slot, lp, comp, rmax, lmax);
            } else {
                int c = contactOf[slA + j];
                C.state[c] = final_state(P, R, slot, lp, slide);
                for (int q = 0; q < 3; q++) C.lam[q * C.cap + c] = (double)lp[q];
            }
        }
        if (op == OP_WARM || op == OP_SWEEP) {
            float2* da = reinterpret_cast<float2*>(dv + 6 * id.x);
            float2* db = reinterpret_cast<float2*>(dv + 6 * id.y);
            if (P.ma != 0.f) for (int q = 0; q < 3; q++) da[q] = make_float2(P.a[2 * q], P.a[2 * q + 1]);
            if (P.mb != 0.f) for (int q = 0; q < 3; q++) db[q] = make_float2(P.b[2 * q], P.b[2 * q + 1]);
        }
        if (op == OP_SWEEP && accel) nncg_acc(gsq, e0, acc);
    };
    // one pass of `op` over the scene, colour by colour.  Resident: the whole
    // scene sits in the buffers and the chunks of one colour run together.
    // Otherwise chunks stream through the two buffers: chunk i + 1 is copied
    // in while chunk i is processed, and (sweeps only) a chunk's multipliers
    // go back to global memory after it.
    // colour heads of the chunk list (bit 30 marks a chunk that starts a colour)
    // (and, for a resident scene, each colour's first group, kept here so a
    // sweep reads no global memory)
    __shared__ int s_head[MAXCB + 1], s_kh[MAXCB + 1];
    __shared__ int s_nhead;
    if (t == 0) {
        int nh = 0;
        for (int i = 0; i < nch; i++)
            if ((ck[i] & HEAD) && nh < MAXCB) s_head[nh++] = i;
        s_head[nh] = nch;
        s_nhead = nh;
        for (int h = 0; h <= nh; h++) s_kh[h] = ck[s_head[h]] & KMASK;
    }
    __syncthreads();
    const int nhead = s_nhead;
    auto pass = [&](int op, bool rev) {
        if (resident) {
            for (int hh = 0; hh < nhead; hh++) {
                int h = rev ? nhead - 1 - hh : hh;
                int k0 = s_kh[h], k1 = s_kh[h + 1];
                for (int k = k0 + t; k < k1; k += T) {
                    int2 gi = sgi[k - kS0];
                    group(op, gi.x - slotS0, gi.x, gi.y, sgl[k - kS0]);
                }
                if (op == OP_SWEEP && accel && hh == nhead - 1) nncg_flush(acc, s_tot[par]);
                __syncthreads();
            }
            return;
        }
        auto chunkAt = [&](int m) { return rev ? nch - 1 - m : m; };
        {
            int i = chunkAt(0);
            stage(0, ck[i] & KMASK, ck[i + 1] & KMASK);
        }
        for (int m = 0; m < nch; m++) {
            int buf = m & 1;
            int i = chunkAt(m);
            int k0 = ck[i] & KMASK, k1 = ck[i + 1] & KMASK;
            if (m + 1 < nch) {
                int i2 = chunkAt(m + 1);
                stage(buf ^ 1, ck[i2] & KMASK, ck[i2 + 1] & KMASK);
                cp_async_wait_one();
            } else {
                cp_async_wait_all();
            }
            __syncthreads();
            const int2* gi0 = sgi + buf * cap;
            const int2* gl0 = sgl + buf * cap;
            int ss = gi0[0].x;
            for (int k = k0 + t; k < k1; k += T) {
                int2 gi = gi0[k - k0];
                group(op, buf * cap + gi.x - ss, gi.x, gi.y, gl0[k - k0]);
            }
            if (op == OP_SWEEP && accel && m == nch - 1) nncg_flush(acc, s_tot[par]);
            __syncthreads();
            if (op == OP_SWEEP) {
                unstage(buf, k0, k1);
                __syncthreads();
            }
        }
    };

    if (resident) {
        stage(0, kS0, kS1);
        cp_async_wait_all();
    }
    __syncthreads();
    int total = 0;
    float res = 0.f;
    // attempt 0 starts from lamS; with lamAlt given, a scene that misses the
    // residual target starts again from lamAlt (the learned start's fallback)
    const int attempts = (lamAlt && check > 0 && tolRel > 0.f) ? 2 : 1;
    for (int attempt = 0; attempt < attempts; attempt++) {
        if (attempt == 1) {
            if (res <= tolRel) break;   // uniform: res comes from shared memory
            if (resident)
                for (int i = t; i < nslots * 4; i += T) slam[4 * lam_pos(i >> 2) + (i & 3)] = lamAlt[(size_t)slotS0 * 4 + i];
            else
                for (int i = t; i < nslots * 4; i += T) lamS[(size_t)slotS0 * 4 + i] = lamAlt[(size_t)slotS0 * 4 + i];
            for (int b = t; b < nbA; b += T)
                for (int k = 0; k < 6; k++) dv[6 * b + k] = 0.f;
            if (t == 0 && sceneFall) sceneFall[s] = 1;
            __syncthreads();
        } else if (t == 0 && sceneFall) {
            sceneFall[s] = 0;
        }
        pass(OP_WARM, false);
        pend = false;
        float ggPrev = 0.f;
        if (accel) {   // delta-v at the first sweep's start, q = 0
            for (int b = t; b < nbA; b += T)
                for (int k = 0; k < 6; k++) {
                    dqB[12 * b + k] = dv[6 * b + k];
                    dqB[12 * b + 6 + k] = 0.f;
                }
            if (t < 2 * NNCG_SCALES) s_tot[t / NNCG_SCALES][t % NNCG_SCALES] = 0ull;
            e0 = nncg_e0(0, 0.f);
            __syncthreads();
        }
        int done = 0;
        for (int it = 0; it < iters; it++) {
            pass(OP_SWEEP, sym && (it & 1));
            done = it + 1;
            if (accel) {
                // |g|^2 from the exact totals, then the momentum step on every
                // slot and every body (no colour order needed)
                const float gg = nncg_gg(s_tot[par], e0);
                const float beta = nncg_beta(it, gg, ggPrev);
                ggPrev = gg;
                if (t < NNCG_SCALES) s_tot[par ^ 1][t] = 0ull;   // the next sweep's totals
                e0 = nncg_e0(1, gg);
                par ^= 1;
                // eager passes where the multipliers are read next (a residual
                // check, the last sweep) or the colours are walked backwards;
                // otherwise the next sweep applies the step as it goes
                const bool eager = sym || done == iters || (check > 0 && done % check == 0);
                if (eager) {
                    for (int i = t; i < nslots; i += T) {
                        float* lp = resident ? slam + 4 * lam_pos(i) : lamS + 4 * ((size_t)slotS0 + i);
                        float* gp = resident ? sgp + 8 * lam_pos(i) : gpG + 8 * ((size_t)slotS0 + i);
                        nncg_slot(lp, gp, it, beta);
                    }
                    // pinned bodies keep delta-v 0 (the lazy path skips them too)
                    for (int b = t; b < nbA; b += T)
                        if (mv[b] != 0.f) nncg_body(dv + 6 * b, dqB + 12 * b, it, beta);
                }
                pend = !eager;
                pendIt = it;
                pendBeta = beta;
                __syncthreads();   // also orders the totals' reset before the next sweep adds to them
            }
            // the same check points as the cluster kernel, so a scene stops at
            // the same sweep whichever kernel solves it
            if (check > 0 && (done % check == 0 || done == iters)) {
                if (t == 0) { s_res = 0.f; s_lam = 0.f; }
                rmax = 0.f;
                lmax = 0.f;
                __syncthreads();
                pass(OP_RES, false);
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
    if (!writeBack) return;   // autotuner trial: results are discarded
    pass(OP_FINAL, false);
    for (int b = t; b < nb; b += T) {
        const int l = lidOf[b0 + b];
        for (int k = 0; k < 6; k++) B.dv[6 * (b0 + b) + k] = l >= 0 ? (double)dv[6 * l + k] : 0.0;
    }
    if (t == 0) {
        sceneSweeps[s] = total;
        sceneRes[s] = res;
        trace_scene(trace, s, tStart);
    }
}

// ---------------------------------------------------------------------------
// Scenes too large for one CTA's shared memory: a thread-block cluster of K
// CTAs (on K SMs) holds one scene.  Every colour's slot range is split into
// K equal windows; CTA `rank` keeps the groups that start in its window, so
// the scene's records stay resident across the cluster for the whole solve.
// Body delta-v is distributed: body b lives in the shared memory of CTA
// b % K (slot b / K) and is read and written through distributed shared
// memory.  A cluster barrier separates colours; residual checks reduce into
// CTA 0.  Every CTA runs the same colour and sweep loops and takes the stop
// decision from the same reduced value, so all of them reach every barrier.
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned dsm_map(const void* p, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ float2 dsm_ld2(unsigned a) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ float4 dsm_ld4(unsigned a) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(a)
                 : "memory");
    return v;
}
__device__ __forceinline__ void dsm_st4(unsigned a, float x, float y, float z, float w) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(x), "f"(y), "f"(z), "f"(w)
                 : "memory");
}
__device__ __forceinline__ void dsm_st2(unsigned a, float x, float y) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(x), "f"(y) : "memory");
}
__device__ __forceinline__ int dsm_ld_s32(unsigned a) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void dsm_st_s32(unsigned a, int v) {
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long dsm_ld_u64(unsigned a) {
    unsigned long long v;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void dsm_max_s32(unsigned a, int v) {
    asm volatile("red.shared::cluster.max.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// With the conjugate-gradient acceleration on, a CTA also keeps per owned
// body delta-v at the sweep's start and q (12 floats) and per staged slot g
// and p (8 floats).
struct ClusterSmem {
    int dv, dq, mv, rec, lam, gp, gi, gl, total;
    __host__ __device__ ClusterSmem(int nbMax, int K, int cap, int accel = 0) {
        int own = (nbMax + K - 1) / K;
        dv = 0;               // 12 floats per owned body: delta-v, then symmetric jinv
        dq = 12 * own;
        mv = dq + (accel ? 12 * own : 0);
        rec = (mv + nbMax + 3) & ~3;
        lam = rec + cap * RECS;
        gp = lam + 4 * cap;
        gi = gp + (accel ? 8 * cap : 0);
        gl = gi + 2 * cap;
        total = gl + 2 * cap;
    }
};

__global__ void __launch_bounds__(256, 1) k_batch_sweep_cluster(
    DBodies B, DContacts C, const int* sceneBodyOff, const int* bigScenes, const int* colOff, const int2* gInfo,
    const int2* glid, const int* contactOf, const float* __restrict__ rec, const float* lamS, int cap, int nbMax,
    int K, int iters, float omega, float comp, float tolRel, int check, float slide, int* sceneSweeps,
    float* sceneRes, int inner, int writeBack, float relax, int sym, long long* trace, const int* lidOf,
    const int* bodyOf, const int* sceneActive, int accel) {
    extern __shared__ float sm[];
    const ClusterSmem L(nbMax, K, cap, accel);
    const long long tStart = gtimer();
    float* dvOwn = sm + L.dv;
    float* mv = sm + L.mv;
    float* srec = sm + L.rec;
    float* slam = sm + L.lam;
    int2* sgi = reinterpret_cast<int2*>(sm + L.gi);
    int2* sgl = reinterpret_cast<int2*>(sm + L.gl);
    __shared__ int s_lo[MAXCB], s_hi[MAXCB], s_gs[MAXCB], s_kb[MAXCB + 1], s_sb[MAXCB + 1];
    __shared__ int s_ok, s_any;          // capacity flags (s_any lives on CTA 0)
    __shared__ int s_resC, s_lamC;       // cluster-wide maxima (CTA 0), float bits
    __shared__ int s_res, s_lam;         // CTA-local maxima, float bits
    const unsigned rank = cluster_rank();
    const int s = bigScenes[blockIdx.x / K];
    const int t = threadIdx.x, T = blockDim.x;
    const int b0 = sceneBodyOff[s], nb = sceneBodyOff[s + 1] - b0;
    const int nbA = sceneActive[s];     // active bodies (compact ids); owner of id b: CTA b % K
    const int own = (nbA + K - 1) / K;
    const int* co = colOff + s * (MAXCB + 1);
    const int ncol = scene_colours(co);
    for (int b = t; b < nbA; b += T) {
        const int gb = bodyOf[b0 + b];
        mv[b] = (B.flags[gb] & F_PINNED) ? 0.f : (float)B.minv[gb];
    }
    for (int i = t; i < own; i += T) {
        int lb = i * K + (int)rank;
        for (int k = 0; k < 6; k++) dvOwn[12 * i + k] = 0.f;
        if (lb < nbA) {
            const int gb = bodyOf[b0 + lb];
            load_jinv(B, gb, (B.flags[gb] & F_PINNED) != 0, dvOwn + 12 * i + 6);
        } else {
            for (int k = 0; k < 6; k++) dvOwn[12 * i + 6 + k] = 0.f;
        }
    }
    // this CTA's part of every colour: groups starting in window `rank`
    for (int col = t; col < ncol; col += T) {
        int k0 = co[col], k1 = co[col + 1];
        int2 e = gInfo[k1 - 1];
        int st = gInfo[k0].x, span = e.x + e.y - st;
        int w0 = st + (int)((long long)span * rank / K), w1 = st + (int)((long long)span * (rank + 1) / K);
        // first group starting at or after w0 (w1): binary search over the
        // colour's ascending group start slots
        int lo = k0, z = k1;
        while (lo < z) { int m = (lo + z) >> 1; if (gInfo[m].x < w0) lo = m + 1; else z = m; }
        int hi = k1;
        if (rank + 1 < (unsigned)K) {
            int a = lo;
            z = k1;
            while (a < z) { int m = (a + z) >> 1; if (gInfo[m].x < w1) a = m + 1; else z = m; }
            hi = a;
        }
        s_lo[col] = lo;
        s_hi[col] = hi;
        s_gs[col] = hi > lo ? gInfo[lo].x : 0;
    }
    if (t == 0) { s_any = 1; s_resC = 0; s_lamC = 0; }
    __syncthreads();
    if (t == 0) {
        int kb = 0, sb = 0;
        for (int col = 0; col < ncol; col++) {
            s_kb[col] = kb;
            s_sb[col] = sb;
            int lo = s_lo[col], hi = s_hi[col];
            kb += hi - lo;
            if (hi > lo) { int2 e = gInfo[hi - 1]; sb += e.x + e.y - gInfo[lo].x; }
        }
        s_kb[ncol] = kb;
        s_sb[ncol] = sb;
        s_ok = (sb <= cap && kb <= cap) ? 1 : 0;
    }
    cluster_sync_all();
    // every CTA learns whether all parts fit; if one does not, all return here
    if (t == 0 && !s_ok) dsm_st_s32(dsm_map(&s_any, 0), 0);
    cluster_sync_all();
    int okAll = dsm_ld_s32(dsm_map(&s_any, 0));
    cluster_sync_all();
    if (!okAll) {
        if (rank == 0 && t == 0) { sceneSweeps[s] = -1; sceneRes[s] = 1e30f; }
        return;
    }
    // stage this CTA's parts of all colours
    for (int col = 0; col < ncol; col++) {
        int lo = s_lo[col], hi = s_hi[col];
        if (hi <= lo) continue;
        int gs0 = gInfo[lo].x;
        int2 e = gInfo[hi - 1];
        int nsl = e.x + e.y - gs0;
        for (int i = t; i < nsl * (REC / 4); i += T) {
            int sl = i / (REC / 4), q = i - sl * (REC / 4);
            int bs = s_sb[col] + sl;   // slot in the staged records
            cp_async16(srec + bs * RECS + 4 * rec_pos(rec_rot(bs), q), rec + (size_t)(gs0 + sl) * REC + 4 * q);
        }
        for (int i = t; i < nsl; i += T) cp_async16(slam + 4 * lam_pos(s_sb[col] + i), lamS + 4 * ((size_t)gs0 + i));
        for (int i = t; i < hi - lo; i += T) {
            cp_async8(sgi + s_kb[col] + i, gInfo + lo + i);
            cp_async8(sgl + s_kb[col] + i, glid + lo + i);
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();

    float* dq = sm + L.dq;
    float* sgp = sm + L.gp;
    // |g|^2 totals of this CTA's groups by sweep parity, and the cluster's
    // totals gathered from every CTA
    __shared__ unsigned long long s_tot[2][NNCG_SCALES], s_all[8 * NNCG_SCALES];
    Acc4 acc;
    int e0 = 0, par = 0;
    float rmax = 0.f, lmax = 0.f;
    // a momentum step left pending by the previous sweep, applied as the
    // one-CTA kernel applies it (each body at its first touch, each slot
    // before its update); a body's dq lives with its owner CTA
    bool pend = false;
    int pendIt = 0;
    float pendBeta = 0.f;
    auto dq_remote = [&](float* v, int b) {
        const unsigned a = dsm_map(dq + 12 * (b / K), b % K);
        float d0[6], q[6];
        dq_unpack(dsm_ld4(a), dsm_ld4(a + 16), dsm_ld4(a + 32), d0, q);
        nncg_body_core(v, d0, q, pendIt, pendBeta);
        dsm_st4(a, d0[0], d0[1], d0[2], d0[3]);
        dsm_st4(a + 16, d0[4], d0[5], q[0], q[1]);
        dsm_st4(a + 32, q[2], q[3], q[4], q[5]);
    };
    auto group = [&](int op, int col, int kk) {
        int2 gi = sgi[kk];
        const int2 idf = sgl[kk];
        const int2 id = make_int2(idf.x & GL_ID, idf.y & GL_ID);
        int sl0 = s_sb[col] + (gi.x - s_gs[col]);
        // each body's delta-v and inverse inertia live with its owner CTA
        unsigned pa = dsm_map(dvOwn + 12 * (id.x / K), id.x % K);
        unsigned pb = dsm_map(dvOwn + 12 * (id.y / K), id.y % K);
        Pair P;
        {
            float4 u0 = dsm_ld4(pa), u1 = dsm_ld4(pa + 16), u2 = dsm_ld4(pa + 32);
            float4 v0 = dsm_ld4(pb), v1 = dsm_ld4(pb + 16), v2 = dsm_ld4(pb + 32);
            P.a[0] = u0.x; P.a[1] = u0.y; P.a[2] = u0.z; P.a[3] = u0.w; P.a[4] = u1.x; P.a[5] = u1.y;
            P.ja[0] = u1.z; P.ja[1] = u1.w; P.ja[2] = u2.x; P.ja[3] = u2.y; P.ja[4] = u2.z; P.ja[5] = u2.w;
            P.b[0] = v0.x; P.b[1] = v0.y; P.b[2] = v0.z; P.b[3] = v0.w; P.b[4] = v1.x; P.b[5] = v1.y;
            P.jb[0] = v1.z; P.jb[1] = v1.w; P.jb[2] = v2.x; P.jb[3] = v2.y; P.jb[4] = v2.z; P.jb[5] = v2.w;
        }
        P.ma = mv[id.x];
        P.mb = mv[id.y];
        const bool lazy = op == OP_SWEEP && pend;
        if (lazy) {
            if ((idf.x & GL_FIRST) && P.ma != 0.f) dq_remote(P.a, id.x);
            if ((idf.y & GL_FIRST) && P.mb != 0.f) dq_remote(P.b, id.y);
        }
        const int cnt = gi.y;
        const int reps = op == OP_SWEEP ? inner : 1;
        float gsq = 0.f;
        for (int jj = 0; jj < reps * cnt; jj++) {
            const int j = reps == 1 ? jj : jj % cnt;
            const int slot = sl0 + j;
            const float* R = srec + slot * RECS;
            float* lp = slam + 4 * lam_pos(slot);
            if (op == OP_WARM) {
                warm_contact(P, R, slot, lp);
            } else if (op == OP_SWEEP) {
                float d[3];
                float4 l = sld4(lp);
                if (lazy && jj < cnt) l = nncg_slot_reg(l, sgp + 8 * lam_pos(slot), pendIt, pendBeta);
                sweep_contact_l(P, R, slot, l, lp, omega, comp, relax, d);
                if (accel) {
                    float* g = sgp + 8 * lam_pos(slot);
                    if (jj >= cnt)
                        for (int q = 0; q < 3; q++) d[q] = __fadd_rn(g[q], d[q]);
                    *reinterpret_cast<float4*>(g) = make_float4(d[0], d[1], d[2], 0.f);
                    if (jj >= (reps - 1) * cnt) gsq = sq3_acc(d, gsq);
                }
            } else if (op == OP_RES) {
                res_contact(P, R, slot, lp, comp, rmax, lmax);
            } else {
                int c = contactOf[gi.x + j];
                C.state[c] = final_state(P, R, slot, lp, slide);
                for (int q = 0; q < 3; q++) C.lam[q * C.cap + c] = (double)lp[q];
            }
        }
        if (op == OP_WARM || op == OP_SWEEP) {
            if (P.ma != 0.f) { dsm_st4(pa, P.a[0], P.a[1], P.a[2], P.a[3]); dsm_st2(pa + 16, P.a[4], P.a[5]); }
            if (P.mb != 0.f) { dsm_st4(pb, P.b[0], P.b[1], P.b[2], P.b[3]); dsm_st2(pb + 16, P.b[4], P.b[5]); }
        }
        if (op == OP_SWEEP && accel) nncg_acc(gsq, e0, acc);
    };
    // colours in order, a cluster barrier after each one that writes delta-v
    auto pass = [&](int op, bool rev) {
        for (int cc = 0; cc < ncol; cc++) {
            int col = rev ? ncol - 1 - cc : cc;
            for (int kk = s_kb[col] + t; kk < s_kb[col + 1]; kk += T) group(op, col, kk);
            if (op == OP_SWEEP && accel && cc == ncol - 1) nncg_flush(acc, s_tot[par]);
            if (op == OP_WARM || op == OP_SWEEP) cluster_sync_all();
        }
    };

    cluster_sync_all();   // zeroed delta-v of every CTA visible before any remote access
    pass(OP_WARM, false);
    if (accel) {   // delta-v of the owned bodies at the first sweep's start
        for (int i = t; i < own; i += T)
            for (int k = 0; k < 6; k++) {
                dq[12 * i + k] = dvOwn[12 * i + k];
                dq[12 * i + 6 + k] = 0.f;
            }
        if (t < 2 * NNCG_SCALES) s_tot[t / NNCG_SCALES][t % NNCG_SCALES] = 0ull;
        e0 = nncg_e0(0, 0.f);
        // every CTA has copied its bodies (and cleared its totals) before any
        // CTA's first sweep writes them
        cluster_sync_all();
    }
    int done = 0;
    float res = 0.f;
    float ggPrev = 0.f;
    for (int it = 0; it < iters; it++) {
        pass(OP_SWEEP, sym && (it & 1));
        done = it + 1;
        if (accel) {
            // every CTA gathers the totals of all CTAs (complete at the last
            // colour's barrier) and adds them in integers, so all get the same
            // beta; then each updates its own slots and bodies
            if (t < K * NNCG_SCALES) s_all[t] = dsm_ld_u64(dsm_map(&s_tot[par][t % NNCG_SCALES], t / NNCG_SCALES));
            __syncthreads();
            unsigned long long tot[NNCG_SCALES];
#pragma unroll
            for (int j = 0; j < NNCG_SCALES; j++) {
                tot[j] = 0ull;
                for (int r = 0; r < K; r++) tot[j] += s_all[r * NNCG_SCALES + j];
            }
            const float gg = nncg_gg(tot, e0);
            const float beta = nncg_beta(it, gg, ggPrev);
            ggPrev = gg;
            if (t < NNCG_SCALES) s_tot[par ^ 1][t] = 0ull;   // the next sweep's totals
            e0 = nncg_e0(1, gg);
            par ^= 1;
            // the one-CTA kernel's rule: eager passes where the multipliers are
            // read next or the colours run backwards, else applied as the next
            // sweep goes
            const bool eager = sym || done == iters || (check > 0 && done % check == 0);
            if (eager) {
                for (int i = t; i < s_sb[ncol]; i += T)
                    nncg_slot(slam + 4 * lam_pos(i), sgp + 8 * lam_pos(i), it, beta);
                // pinned bodies (and padding) keep delta-v 0, as in the lazy path
                for (int i = t; i < own; i += T) {
                    const int lb = i * K + (int)rank;
                    if (lb < nbA && mv[lb] != 0.f) nncg_body(dvOwn + 12 * i, dq + 12 * i, it, beta);
                }
                // delta-v of every CTA updated before anyone reads it again
                cluster_sync_all();
            } else {
                __syncthreads();   // this CTA's totals reset before its next additions
            }
            pend = !eager;
            pendIt = it;
            pendBeta = beta;
        }
        if (check > 0 && (done % check == 0 || done == iters)) {
            if (t == 0) { s_res = 0; s_lam = 0; }
            rmax = 0.f;
            lmax = 0.f;
            __syncthreads();
            pass(OP_RES, false);
            atomicMax(&s_res, __float_as_int(rmax));
            atomicMax(&s_lam, __float_as_int(lmax));
            __syncthreads();
            if (t == 0) {
                dsm_max_s32(dsm_map(&s_resC, 0), s_res);
                dsm_max_s32(dsm_map(&s_lamC, 0), s_lam);
            }
            cluster_sync_all();
            float rr = __int_as_float(dsm_ld_s32(dsm_map(&s_resC, 0)));
            float ll = __int_as_float(dsm_ld_s32(dsm_map(&s_lamC, 0)));
            res = rr / fmaxf(1.f, ll);
            cluster_sync_all();   // everyone has read CTA 0's maxima
            if (rank == 0 && t == 0) { s_resC = 0; s_lamC = 0; }
            if (res <= tolRel) break;
        }
    }
    if (writeBack) {   // an autotuner trial discards its results
        pass(OP_FINAL, false);
        // owners write their bodies' delta-v back; CTA 0 clears the bodies
        // without contacts
        for (int i = t; i < own; i += T) {
            int lb = i * K + (int)rank;
            if (lb < nbA) {
                const int gb = bodyOf[b0 + lb];
                for (int k = 0; k < 6; k++) B.dv[6 * gb + k] = (double)dvOwn[12 * i + k];
            }
        }
        if (rank == 0)
            for (int b = t; b < nb; b += T)
                if (lidOf[b0 + b] < 0)
                    for (int k = 0; k < 6; k++) B.dv[6 * (b0 + b) + k] = 0.0;
        if (rank == 0 && t == 0) {
            sceneSweeps[s] = done;
            sceneRes[s] = res;
            trace_scene(trace, s, tStart);
        }
    }
    cluster_sync_all();   // no CTA leaves while another may still read its shared memory
}

size_t batch_cluster_smem(int nbMax, int K, int cap, int accel) {
    return sizeof(float) * (size_t)ClusterSmem(nbMax, K, cap, accel).total;
}

const void* batch_sweep_kernel() { return (const void*)k_batch_sweep; }

size_t batch_sweep_smem(int nbMax, int cap, int accel) { return sizeof(float) * (size_t)SweepSmem(nbMax, cap, accel).total; }

int Ctx::batchLaunchSweep(int threads, int cap, int iters, float tol, int check, float* lamStart, const float* lamAlt,
                          int* fall, int writeBack, int nGrid, const int* order, int nbMax, cudaStream_t strm) {
    double comp = P.enable_compliance ? P.compliance : 0.;
    size_t ssm = batch_sweep_smem(nbMax, cap, batchAccel);
    if (nGrid <= 0) return AM_OK;
    k_batch_sweep<<<nGrid, threads, ssm, strm>>>(
        B, C[cur], sceneBodyOffDev, order, bGInfo, bLid, bChunkK, bNChunks, bContactOf, bRec, lamStart, cap,
        nbMax, iters, (float)P.omega, (float)comp, tol, check, (float)P.sliding_threshold, bSweeps, bRes,
        lamAlt, fall, writeBack, batchInner, (float)batchRelax, batchSym, writeBack ? bTrace : nullptr, bLidOf, bBodyOf,
        bSceneActive, batchAccel, bGP, bDQ);
    AM_LAUNCHED(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("sweep launch: ") + cudaGetErrorString(e); return AM_E_CUDA; }
    return AM_OK;
}

// The split of the scenes for the sweep with staging capacity `cap`: a scene
// whose records fit the one-CTA kernel's two buffers stays there; a larger one
// goes to the cluster kernel with the smallest K in {2, 4, 8} whose CTAs can
// hold it (its slots / K plus one group per colour within each CTA's
// capacity), otherwise it streams through the one-CTA kernel.  Small scenes
// that fit a size class go to that class's launch instead, whose CTAs are
// sized for the class, so several of them share an SM.  Every list is
// ordered costliest first (contacts x sweeps of the previous step) and they
// are stored one after another: one-CTA scenes, the size classes, then
// clusters of 2, 4 and 8.  Each launch lays out shared memory for the most
// bodies among its scenes (and a cluster launch for its largest part).
static const int CLUSTER_K[3] = {2, 4, 8};
// Size classes of resident scenes: staging capacity (a scene of at most
// 2 x cap slots and 4 x cap bodies whose layout fits shared memory) and CTA
// size of each class launch.
static const int NCLASS = 10;
static const int CLASS_CAP[NCLASS] = {16, 32, 64, 128, 192, 256, 384, 512, 576, 640};
static const int CLASS_THREADS[NCLASS] = {32, 32, 64, 128, 192, 256, 384, 512, 512, 512};

int Ctx::batchSplit(int cap, bool useCluster) {
    int S = nScenes;
    hSmall.clear();
    for (auto& v : hBigK) v.clear();
    for (auto& v : hClass) v.clear();
    std::vector<int2> sz(S);
    std::vector<int> act(S);
    cudaMemcpyAsync(sz.data(), bSceneSize, sizeof(int2) * S, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(act.data(), bSceneActive, sizeof(int) * S, cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    smallNb = 0;
    for (int q = 0; q < NCLASS; q++) classNb[q] = 0;
    auto costOf = [&](int sc) { return (size_t)sc < lastCost.size() ? lastCost[sc] : 0; };
    long long costTop = 0;
    for (long long c : lastCost) costTop = std::max(costTop, c);
    for (int q = 0; q < 3; q++) { bigNb[q] = 0; bigCap[q] = 0; }
    for (int sc = 0; sc < S; sc++) {
        const int nb = act[sc], slots = sz[sc].x;   // active bodies: the ones the sweep keeps
        // the smallest size class that holds the scene resident (a scene
        // without contacts touches no shared memory: the smallest class)
        int c = -1;
        if (batchClasses)
            for (int q = 0; q < NCLASS && c < 0; q++)
                if (slots == 0 || (slots <= 2 * CLASS_CAP[q] && nb <= 4 * CLASS_CAP[q] &&
                                   batch_sweep_smem(nb, CLASS_CAP[q], batchAccel) <= batchSmemLimit))
                    c = q;
        if (c >= 0) {
            hClass[c].push_back(sc);
            if (slots > 0) classNb[c] = std::max(classNb[c], nb);
            continue;
        }
        if (useCluster && (batchClasses || slots > 2 * cap)) {
            int need = -1;
            // the smallest cluster whose launch, with this scene added, still
            // fits shared memory (the launch lays out its most bodies and its
            // largest part).  A scene among the longest solves of the last
            // step (cost at least 3/4 of the largest) holds at most 640
            // records per CTA: a sweep takes less time the fewer records each
            // CTA holds, and these scenes bound the whole solve.
            const bool critical = costTop > 0 && (double)costOf(sc) >= batchCriticalFrac * (double)costTop;
            const int capK = critical ? std::min(clusterCap, batchCriticalCap) : clusterCap;
            for (int q = 0; q < 3; q++) {
                int K = CLUSTER_K[q];
                int per = ((slots + K - 1) / K + sz[sc].y + 31) & ~31;
                if (per <= capK && batch_cluster_smem(std::max(bigNb[q], nb), K, std::max(bigCap[q], per), batchAccel) <=
                                             clusterSmemLimit) {
                    need = q;
                    hBigK[q].push_back(sc);
                    bigNb[q] = std::max(bigNb[q], nb);
                    bigCap[q] = std::max(bigCap[q], per);
                    break;
                }
            }
            if (need >= 0) continue;
        }
        hSmall.push_back(sc);
        if (slots > 0) smallNb = std::max(smallNb, nb);
    }
    auto byCost = [&](int a, int b) {
        long long ca = (size_t)a < lastCost.size() ? lastCost[a] : 0, cb = (size_t)b < lastCost.size() ? lastCost[b] : 0;
        return ca > cb;
    };
    std::vector<int> all;
    std::stable_sort(hSmall.begin(), hSmall.end(), byCost);
    all.insert(all.end(), hSmall.begin(), hSmall.end());
    for (auto& v : hClass) {
        std::stable_sort(v.begin(), v.end(), byCost);
        all.insert(all.end(), v.begin(), v.end());
    }
    for (auto& v : hBigK) {
        std::stable_sort(v.begin(), v.end(), byCost);
        all.insert(all.end(), v.begin(), v.end());
    }
    cudaMemcpyAsync(bSceneOrderBuf, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, stream);
    return syncErr();
}

int Ctx::batchClusterScenes() const {
    int n = 0;
    for (auto& v : hBigK) n += (int)v.size();
    return n;
}

int Ctx::batchClusterMaxK() const {
    int k = 0;
    for (int q = 0; q < 3; q++)
        if (!hBigK[q].empty()) k = CLUSTER_K[q];
    return k;
}

// CTAs that solved each scene in the last split: 1 for the one-CTA launch
// and the size classes, K for a cluster of K
void Ctx::batchSceneCtas(int* out) const {
    for (int s = 0; s < nScenes; s++) out[s] = 1;
    for (int q = 0; q < 3; q++)
        for (int s : hBigK[q]) out[s] = CLUSTER_K[q];
}

// the cluster launch of cluster size CLUSTER_K[q] over `list`
int Ctx::batchLaunchCluster(int q, const int* list, int nBig, cudaStream_t strm, int iters, float tol, int check,
                            int writeBack) {
    double comp = P.enable_compliance ? P.compliance : 0.;
    int K = CLUSTER_K[q];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nBig * K);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = batch_cluster_smem(bigNb[q], K, bigCap[q], batchAccel);
    cfg.stream = strm;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = K;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_sweep_cluster, B, C[cur], (const int*)sceneBodyOffDev, list,
                                       (const int*)bColOff, (const int2*)bGInfo, (const int2*)bLid,
                                       (const int*)bContactOf, (const float*)bRec, (const float*)bLam, bigCap[q],
                                       bigNb[q], K, iters, (float)P.omega, (float)comp, tol, check,
                                       (float)P.sliding_threshold, bSweeps, bRes, batchInner, writeBack,
                                       (float)batchRelax, batchSym, writeBack ? bTrace : nullptr, (const int*)bLidOf,
                                       (const int*)bBodyOf, (const int*)bSceneActive, batchAccel);
    AM_LAUNCHED(1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("cluster sweep launch: ") + cudaGetErrorString(e); return AM_E_CUDA; }
    return AM_OK;
}

// Every launch of the solve (the one-CTA kernel, the size classes, the
// cluster sizes) on its own stream, forked from and joined back into the
// context stream.  A scene's solve time is about its sweeps x (1024 +
// contacts) of the previous step (the cost).  Each launch's list (costliest
// first) is cut in two: the scenes within 40 % of the largest cost of the
// batch, which bound the solve and must start at once, and the rest.  The
// first parts of all launches are issued before the second parts, each group
// costliest launch first, on streams of descending priority, so the CTA
// scheduler starts the long solves first across launches.
int Ctx::batchLaunchAll(int threads, int cap, int iters, float tol, int check, float* lamStart, const float* lamAlt,
                        int writeBack) {
    struct L { int kind, q, n, tier; const int* list; long long cost; };
    std::vector<L> ls;
    long long top = 0;
    for (long long c : lastCost) top = std::max(top, c);
    const long long cut = (top * 2) / 5;
    auto costAt = [&](int sc) { return (size_t)sc < lastCost.size() ? lastCost[sc] : 0; };
    const int* list = bSceneOrderBuf;
    auto add = [&](int kind, int q, const std::vector<int>& v) {
        int n = (int)v.size(), n0 = 0;
        while (n0 < n && costAt(v[n0]) >= cut) n0++;
        if (n0 > 0) ls.push_back({kind, q, n0, 0, list, costAt(v[0])});
        if (n > n0) ls.push_back({kind, q, n - n0, 1, list + n0, costAt(v[n0])});
        list += n;
    };
    add(0, 0, hSmall);
    for (int q = 0; q < NCLASS; q++) add(1, q, hClass[q]);
    for (int q = 0; q < 3; q++) add(2, q, hBigK[q]);
    std::stable_sort(ls.begin(), ls.end(), [](const L& a, const L& b) {
        return a.tier != b.tier ? a.tier < b.tier : a.cost > b.cost;
    });
    if ((int)ls.size() > NPOOL) { err = "too many sweep launches"; return AM_E_STATE; }
    cudaEventRecord(evFork, stream);
    int* fall = writeBack ? bFall : nullptr;
    for (size_t i = 0; i < ls.size(); i++) {
        cudaStream_t st = pool[i];
        cudaStreamWaitEvent(st, evFork, 0);
        int r;
        const L& l = ls[i];
        if (l.kind == 0)
            r = batchLaunchSweep(threads, cap, iters, tol, check, lamStart, lamAlt, fall, writeBack, l.n, l.list,
                                 smallNb, st);
        else if (l.kind == 1)
            r = batchLaunchSweep(CLASS_THREADS[l.q], CLASS_CAP[l.q], iters, tol, check, lamStart, lamAlt, fall,
                                 writeBack, l.n, l.list, classNb[l.q], st);
        else
            r = batchLaunchCluster(l.q, l.list, l.n, st, iters, tol, check, writeBack);
        if (r) return r;
    }
    for (size_t i = 0; i < ls.size(); i++) {
        cudaEventRecord(poolJoin[i], pool[i]);
        cudaStreamWaitEvent(stream, poolJoin[i], 0);
    }
    return AM_OK;
}

// slots and chunks for staging capacity `cap`, then the packed records
int Ctx::batchLayout(int cap) {
    double comp = P.enable_compliance ? P.compliance : 0.;
    int nc = nContacts;
    k_batch_slots<<<nScenes, 256, sizeof(int) * (size_t)maxSceneBodies, stream>>>(
        C[cur], PR, bPairOff, bOrder, bColOff, sceneBodyOffDev, nc, nPairs, cap, bGInfo, bLid, bSlotOf, bContactOf,
        bChunkK, bNChunks, bSceneSize, bLidOf, bBodyOf, bSceneActive, dc);
    k_batch_pack<<<(nc + 127) / 128, 128, 0, stream>>>(B, C[cur], nc, bSlotOf, comp, P.friction_override, P.friction,
                                                     bRec, bLam);
    AM_LAUNCHED(2);
    return AM_OK;
}

int Ctx::batchSolve(double dt) {
    int r;
    int nc = nContacts, np = nPairs, S = nScenes;
    if (nc <= 0) return AM_OK;
    launch_solve_prep(B, C[cur], nc, dt, P.feedback_stiffness, false, P.restitution_override, P.restitution,
                      P.warm_start ? 1 : 0, stream);
    if (nc > bRecCap) {
        int cap = std::max(nc + nc / 2, 4096);
        if (alloc(&bRec, (size_t)REC * cap) || alloc(&bLam, 4 * (size_t)cap) || alloc(&bLamL, 4 * (size_t)cap) ||
            alloc(&bSlotOf, cap) || alloc(&bContactOf, cap) || alloc(&bGP, 8 * (size_t)cap))
            return AM_E_CUDA;
        bRecCap = cap;
    }
    if (np > bPairCap) {
        int cap = std::max(np + np / 2, 4096);
        if (alloc(&bColour, cap) || alloc(&bOrder, cap) || alloc(&bLid, cap) || alloc(&bGInfo, cap)) return AM_E_CUDA;
        bPairCap = cap;
    }
    k_scene_ranges<<<(np + 1 + 255) / 256, 256, 0, stream>>>(PR, np, sceneOfDev, S, bPairOff);
    size_t csm = 2 * sizeof(unsigned long long) * (size_t)maxSceneBodies;
    k_batch_colour<<<S, 256, csm, stream>>>(B, C[cur], PR, bPairOff, sceneBodyOffDev, bColour, bOrder, bColOff,
                                            maxSceneBodies, dc);
    AM_LAUNCHED(2);
    // tune on the first solve and again whenever the contact count has grown
    // by half since the last tuning (piles forming change the best shape);
    // a CTA size and staging capacity both given by the caller are used as is
    if (batchThreadsUser && batchCapUser) {
        batchThreads = batchThreadsUser;
        batchCap = batchCapUser;
    } else if ((batchThreads == 0 || batchCap == 0 || 2 * (long long)nc > 3 * (long long)batchTunedContacts) &&
               (r = batchAutotune(dt))) {
        return r;
    }
    int threads = batchThreads, cap = batchCap;
    if ((r = batchLayout(cap))) return r;
    if ((r = batchSplit(cap, clusterEnabled))) return r;
    bSceneOrder = bSceneOrderBuf;
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
    // scenes too large for one CTA run as clusters on their own streams,
    // concurrently with the one-CTA kernel.  The learned start and its
    // in-kernel fallback apply to the one-CTA scenes; clusters keep the plain
    // previous-frame start.
    if ((r = batchLaunchAll(threads, cap, P.iterations, (float)batchTol, batchCheck, lamStart, lamAlt, 1))) return r;
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

// critical path of one sweep of each scene, in contacts: the sum over its
// colours of the longest group (a group's contacts update one after another,
// and a colour ends when its longest group does); one warp per scene
__global__ void k_scene_chain(const int2* gInfo, const int* colOff, int nScenes, int* chain) {
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (s >= nScenes) return;
    const int* co = colOff + s * (MAXCB + 1);
    const int ncol = scene_colours(co);
    int sum = 0;
    for (int c = 0; c < ncol; c++) {
        int m = 0;
        for (int k = co[c] + lane; k < co[c + 1]; k += 32) m = max(m, gInfo[k].y);
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        sum += m;
    }
    if (lane == 0) chain[s] = sum;
}

int Ctx::batchChain(int* out) {
    if (!bChain && alloc(&bChain, nScenes)) return AM_E_CUDA;
    if (nContacts <= 0 || !bGInfo) {
        for (int s = 0; s < nScenes; s++) out[s] = 0;
        return AM_OK;
    }
    k_scene_chain<<<(nScenes + 7) / 8, 256, 0, stream>>>(bGInfo, bColOff, nScenes, bChain);
    AM_LAUNCHED(1);
    cudaMemcpyAsync(out, bChain, sizeof(int) * nScenes, cudaMemcpyDeviceToHost, stream);
    return syncErr();
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
    int conv = 0, fall = 0, resid = 0;
    for (int s : hSmall) {
        long long ncs = sw[s] > 0 ? cs[s] / sw[s] : 0;
        resid += (ncs > 0 && ncs <= 2 * batchCap) ? 1 : 0;
    }
    for (auto& v : hClass)
        for (int s : v) resid += (sw[s] > 0 && cs[s] > 0) ? 1 : 0;
    for (int s = 0; s < nScenes; s++) {
        tot += sw[s];
        mx = std::max(mx, sw[s]);
        rmax = std::max(rmax, rs[s]);
        conv += rs[s] <= batchTol ? 1 : 0;
        fall += fl[s];
    }
    lFallbackScenes = lUse ? fall : 0;
    batchResident = resid;
    batchSweepsTotal = tot;
    batchContactSweepsLast = 0;
    for (long long v : cs) batchContactSweepsLast += v;
    // expected solve time of every scene orders the next solve's launches:
    // sweeps x (1024 + contacts), as the time of a sweep grows slowly with
    // the scene's size
    lastCost.assign(nScenes, 0);
    for (int sc = 0; sc < nScenes; sc++)
        if (sw[sc] > 0) lastCost[sc] = cs[sc] + 1024LL * sw[sc];
    for (int sc = 0; sc < nScenes; sc++)
        if (sw[sc] < 0) { err = "a scene did not fit its cluster"; return AM_E_CAPACITY; }
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
    std::vector<double> bbox;   // am_scene.bbox of every scene, NaN (derived) where a scene has none
    bool anyBox = false;
    for (int s = 0; s < n; s++) anyBox = anyBox || sc[s].bbox;
    int nodeBase = 0;
    maxSceneBodies = 0;
    for (int s = 0; s < n; s++) {
        const am_scene& a = sc[s];
        if (anyBox)
            for (int k = 0; k < 6 * a.n_bodies; k++) bbox.push_back(a.bbox ? a.bbox[k] : NAN);
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
    all.bbox = anyBox ? bbox.data() : nullptr;
    all.n_subs = 0;   // composite bodies are refused before this point
    all.sub_parent = all.sub_type = nullptr;
    all.sub_shape = all.sub_R = all.sub_t = nullptr;
    int r = setScene(all);
    if (r) return r;
    nScenes = n;
    int cap = host.cap;
    std::vector<int> sOf(cap, n), tEnd(all.n_bodies);
    for (int i = 0; i < all.n_bodies; i++) { sOf[i] = sceneOf[i]; tEnd[i] = bodyOff[sceneOf[i] + 1]; }
    bCS = nullptr;
    if (alloc(&sceneOfDev, cap) || alloc(&sceneBodyOffDev, n + 1) || alloc(&topEnd, all.n_bodies) ||
        alloc(&bPairOff, n + 1) || alloc(&bColOff, (size_t)n * (MAXCB + 1)) || alloc(&bSweeps, n) || alloc(&bRes, n) ||
        alloc(&bFall, n) || alloc(&bTrace, 3 * (size_t)n) || alloc(&bSceneActive, n) ||
        alloc(&bLidOf, (size_t)bodyOff[n] + 1) || alloc(&bBodyOf, (size_t)bodyOff[n] + 1) ||
        alloc(&bDQ, 12 * ((size_t)bodyOff[n] + 1)))
        return AM_E_CUDA;
    cudaMemsetAsync(bFall, 0, sizeof(int) * n, stream);
    cudaMemsetAsync(bTrace, 0, sizeof(long long) * 3 * n, stream);
    cudaMemcpyAsync(sceneOfDev, sOf.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(sceneBodyOffDev, bodyOff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(topEnd, tEnd.data(), sizeof(int) * all.n_bodies, cudaMemcpyHostToDevice, stream);
    if (alloc(&bChunkK, (size_t)n * (MAXCH + 1)) || alloc(&bNChunks, n) || alloc(&bSceneOrderBuf, n) ||
        alloc(&bSceneSize, n))
        return AM_E_CUDA;
    bSceneOrder = nullptr;
    lastCost.clear();
    // streams of the sweep launches, in descending priority (the costliest
    // launch of a solve takes the first)
    int prLeast = 0, prGreatest = 0;
    cudaDeviceGetStreamPriorityRange(&prLeast, &prGreatest);
    for (int q = 0; q < NPOOL; q++) {
        int pr = std::min(prLeast, prGreatest + q);
        if (!pool[q] && cudaStreamCreateWithPriority(&pool[q], cudaStreamNonBlocking, pr) != cudaSuccess) {
            err = "sweep stream";
            return AM_E_CUDA;
        }
        if (!poolJoin[q]) cudaEventCreateWithFlags(&poolJoin[q], cudaEventDisableTiming);
    }
    if (!evFork) cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming);
    // dynamic shared memory the sweep may take: the opt-in limit less its static part
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, batch_sweep_kernel()) != cudaSuccess) { err = "sweep kernel attributes"; return AM_E_CUDA; }
    batchSmemLimit = (size_t)optin > fa.sharedSizeBytes ? optin - fa.sharedSizeBytes : 0;
    if (cudaFuncSetAttribute(batch_sweep_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batchSmemLimit) !=
        cudaSuccess) {
        err = "sweep kernel shared-memory limit";
        return AM_E_CUDA;
    }
    // every sweep launch asks for the largest shared-memory carveout, so CTAs
    // of the size classes and clusters can share an SM
    cudaFuncSetAttribute(batch_sweep_kernel(), cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute((const void*)k_batch_sweep_cluster, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    // cluster kernel: the largest staging capacity (multiple of 32, at most
    // 2048 records) that fits
    cudaFuncAttributes fc;
    clusterUsable = false;
    if (cudaFuncGetAttributes(&fc, (const void*)k_batch_sweep_cluster) == cudaSuccess) {
        size_t lim = (size_t)optin > fc.sharedSizeBytes ? optin - fc.sharedSizeBytes : 0;
        clusterSmemLimit = lim;
        // the most records a CTA of a cluster may hold (a scene's part; its
        // bodies are checked when the scenes are split)
        clusterCap = clusterCapUser > 0 ? clusterCapUser : 2048;
        while (clusterCap > 64 && batch_cluster_smem(64, 2, clusterCap, 0) > lim) clusterCap -= 32;
        if (batch_cluster_smem(64, 2, clusterCap, 0) <= lim &&
            cudaFuncSetAttribute((const void*)k_batch_sweep_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)lim) == cudaSuccess)
            clusterUsable = true;
    }
    clusterEnabled = clusterAllowed && clusterUsable;
    size_t lsm = sizeof(int) * (size_t)maxSceneBodies;
    if (lsm > 40 * 1024 &&
        cudaFuncSetAttribute((const void*)k_batch_slots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm) !=
            cudaSuccess) {
        err = "a scene has too many bodies for the batched slot layout's shared memory";
        return AM_E_CAPACITY;
    }
    size_t csm = 2 * sizeof(unsigned long long) * (size_t)maxSceneBodies;
    if (csm > 40 * 1024 &&   // the kernel's static shared memory (4.4 KB) counts against the 48 KB default
        cudaFuncSetAttribute((const void*)k_batch_colour, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm) !=
            cudaSuccess) {
        err = "a scene has too many bodies for the batched colouring's shared memory";
        return AM_E_CAPACITY;
    }
    return syncErr();
}

// Picks the CTA size and staging capacity of the scene solve: every
// candidate lays out the records for its capacity and runs a few sweeps from
// the same packed state (multipliers restored between candidates); the
// fastest wins.
int Ctx::batchAutotune(double dt) {
    (void)dt;
    const int fixedThreads = batchThreadsUser;   // a CTA size given by the caller is kept
    std::vector<int> thr = fixedThreads > 0 ? std::vector<int>{fixedThreads} : std::vector<int>{128, 256, 512};
    std::vector<int> caps;
    for (int c : {64, 128, 192, 256})
        if (batch_sweep_smem(maxSceneBodies, c, batchAccel) <= batchSmemLimit && (!batchCapUser || c == batchCapUser))
            caps.push_back(c);
    if (batchCapUser && caps.empty() && batch_sweep_smem(maxSceneBodies, batchCapUser, batchAccel) <= batchSmemLimit)
        caps.push_back(batchCapUser);
    if (caps.empty()) {
        err = "a scene has too many bodies for the batched solve's shared memory";
        return AM_E_CAPACITY;
    }
    int nc = nContacts;
    int r0 = 0;
    // With the size classes on, the one-CTA launch only gets scenes that fit
    // no class and no cluster (streamed through its staging buffers).  When
    // there are none at the largest capacity there is nothing to tune.
    if (batchClasses && !fixedThreads) {
        batchLayout(caps.back());
        if ((r0 = batchSplit(caps.back(), clusterEnabled))) return r0;
        if (hSmall.empty()) {
            batchThreads = 256;
            batchCap = caps.back();
            batchTunedContacts = nc;
            return syncErr();
        }
    }
    float* save = bLamL;   // the learned start is written only after tuning
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bestT = 256, bestC = caps[0];
    for (int cap : caps) {
        batchLayout(cap);
        // time the one-CTA kernel on the scenes it would get with this capacity
        if ((r0 = batchSplit(cap, clusterEnabled))) return r0;
        cudaMemcpyAsync(save, bLam, sizeof(float) * 4 * nc, cudaMemcpyDeviceToDevice, stream);
        for (int T : thr) {
            cudaMemcpyAsync(bLam, save, sizeof(float) * 4 * nc, cudaMemcpyDeviceToDevice, stream);
            cudaEventRecord(e0, stream);
            int r = batchLaunchAll(T, cap, 8, 0.f, 0, bLam, nullptr, 0);
            if (r) return r;
            cudaEventRecord(e1, stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; bestT = T; bestC = cap; }
        }
        cudaMemcpyAsync(bLam, save, sizeof(float) * 4 * nc, cudaMemcpyDeviceToDevice, stream);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    batchThreads = bestT;
    batchCap = bestC;
    batchTunedContacts = nc;
    return syncErr();
}

// RigidBodySystem.advanceTime for every scene of the batch (merging off)
int Ctx::stepBatch(double dt) {
    int r;
    if (!evPh[0])
        for (auto& e : evPh) cudaEventCreate(&e);
    if (evA != evPh[3]) {   // the sweep's timing events are phase boundaries 3 and 4
        if (evA) { cudaEventDestroy(evA); cudaEventDestroy(evB); }
        evA = evPh[3];
        evB = evPh[4];
    }
    cudaEventRecord(evPh[0], stream);
    if ((r = beginStep(0))) return r;
    double t = phaseNow();
    if ((r = collisionDetection())) return r;
    phaseAdd(AM_PHASE_DETECTION, t);
    cudaEventRecord(evPh[1], stream);
    t = phaseNow();
    if ((r = warmStart())) return r;
    phaseAdd(AM_PHASE_WARMSTART, t);
    if ((r = wake())) return r;
    cudaEventRecord(evPh[2], stream);
    t = phaseNow();
    // the solve records evA (= evPh[3]) before its sweep launches and evB
    // (= evPh[4]) after them; a step without contacts records both here
    if ((r = batchSolve(dt))) return r;
    phaseAdd(AM_PHASE_LCP_SOLVE, t);
    if (!pgsPending) {
        cudaEventRecord(evPh[3], stream);
        cudaEventRecord(evPh[4], stream);
    }
    if ((r = finishStep(dt))) return r;
    cudaEventRecord(evPh[5], stream);
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
    cudaEventRecord(evPh[6], stream);
    cudaEventSynchronize(evPh[6]);
    for (int k = 0; k < AM_STEP_PHASES; k++) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, evPh[k], evPh[k + 1]) == cudaSuccess) phaseDevMs[k] += ms;
    }
    perf.contact_sweeps += batchContactSweepsLast;
    perf.steps++;
    stats.n_contacts = nContacts;
    return AM_OK;
}

}  // namespace am
