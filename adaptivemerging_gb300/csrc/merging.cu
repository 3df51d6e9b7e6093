// merging.cu -- the step with adaptive merging enabled.
//
// Split of work (the reference keeps its merging logic in the caller,
// Merging.java / RigidCollection.java / BodyPairContact.java; the drop-in
// keeps those decisions on the host and moves every per-contact and per-body
// computation to the device):
//   host   : body-pair contacts (insertion-ordered, the deterministic stand-in
//            for the reference's identity-hashed sets), per-body pair sets,
//            merge / unmerge predicates and collection mass properties,
//            the breadth-first contact order of the single sweep;
//   device : collision, warm start, the single sweep (bit-exact kernel over a
//            gathered contact list), the full solve, motion metrics,
//            integration, sleeping, and the store of contacts that live
//            inside collections.
// Contact references on the host: r >= 0 is contact r of the current step's
// buffer; r < 0 is slot ~r of the collection contact store.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

// ---------------------------------------------------------------------------
// device helpers
// copy whole contacts (all persistent fields) src[si[k]] -> dst[di[k]]
// mode 0: plain copy; mode 1: Contact(Contact) copy constructor semantics
// (newThisTimeStep = false, warm-start copies and b/D zeroed,
// RigidCollection.addToInternalContact, RigidCollection.java:836-847);
// mode 2: lambda / state / Jacobian only (single-sweep scatter);
// mode 3: full copy with lambdaXwarm = lambdaX (contacts handed back to the
// collision processor by unmerge, Merging.java:348-355)
__global__ void k_copy_contacts(DContacts S, const int* si, DContacts D, const int* di, int n, int mode) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int s = si[k], d = di[k];
    int sc = S.cap, dcap = D.cap;
    for (int r = 0; r < 3; r++) D.lam[r * dcap + d] = S.lam[r * sc + s];
    D.state[d] = S.state[s];
    for (int q = 0; q < 36; q++) D.J[q * dcap + d] = S.J[q * sc + s];
    if (mode == 2) return;
    D.b1[d] = S.b1[s]; D.b2[d] = S.b2[s]; D.bv1[d] = S.bv1[s]; D.bv2[d] = S.bv2[s]; D.info[d] = S.info[s];
    D.sb1[d] = S.sb1[s]; D.sb2[d] = S.sb2[s]; D.pair[d] = S.pair[s];
    for (int q = 0; q < 12; q++) D.f[q * dcap + d] = S.f[q * sc + s];
    D.cv[d] = S.cv[s]; D.pcv[d] = S.pcv[s];
    if (mode == 1) {
        D.fresh[d] = 0;
        for (int r = 0; r < 3; r++) D.lamw[r * dcap + d] = 0.0;
        for (int r = 0; r < 6; r++) D.bD[r * dcap + d] = 0.0;
    } else if (mode == 3) {
        D.fresh[d] = S.fresh[s];
        for (int r = 0; r < 3; r++) D.lamw[r * dcap + d] = S.lam[r * sc + s];
        for (int r = 0; r < 6; r++) D.bD[r * dcap + d] = S.bD[r * sc + s];
    } else {
        D.fresh[d] = S.fresh[s];
        for (int r = 0; r < 3; r++) D.lamw[r * dcap + d] = S.lamw[r * sc + s];
        for (int r = 0; r < 6; r++) D.bD[r * dcap + d] = S.bD[r * sc + s];
    }
}

// Contact.computeJacobian(boolean) (Contact.java:235-271): frame from body 1's
// current transform, lever arms from the solve bodies; only contacts touching
// a collection member are recomputed (updateJacobiansThatNeedUpdating,
// CollisionProcessor.java:326-334)
__global__ void k_recompute_J(DBodies B, DContacts C, int n, int inColl) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    int b1 = C.b1[c], b2 = C.b2[c];
    int p1 = B.parent[b1], p2 = B.parent[b2];
    if (p1 < 0 && p2 < 0) return;
    int cap = C.cap;
    m3 R = ldm(B.R + 9 * b1);
    v3 x = ldv(B.x + 3 * b1);
    auto fr = [&](int q) { return mk(C.f[(3 * q) * cap + c], C.f[(3 * q + 1) * cap + c], C.f[(3 * q + 2) * cap + c]); };
    v3 pW = tpoint(R, x, fr(0));
    v3 nn = mxv(R, fr(1)), t1 = mxv(R, fr(2)), t2 = mxv(R, fr(3));
    int s1 = (p1 >= 0 && !inColl) ? p1 : b1;
    int s2 = (p2 >= 0 && !inColl) ? p2 : b2;
    v3 r1 = sub(pW, ldv(B.x + 3 * s1));
    v3 r2 = sub(pW, ldv(B.x + 3 * s2));
    v3 rows[12];
    rows[0] = scale(-1, nn); rows[1] = cross(nn, r1); rows[2] = nn; rows[3] = cross(r2, nn);
    rows[4] = scale(-1, t1); rows[5] = cross(t1, r1); rows[6] = t1; rows[7] = cross(r2, t1);
    rows[8] = scale(-1, t2); rows[9] = cross(t2, r1); rows[10] = t2; rows[11] = cross(r2, t2);
    for (int q = 0; q < 12; q++) {
        C.J[(3 * q) * cap + c] = rows[q].x;
        C.J[(3 * q + 1) * cap + c] = rows[q].y;
        C.J[(3 * q + 2) * cap + c] = rows[q].z;
    }
}

// solve bodies of the full solve: the collection when merged (PGS.java:108-109)
__global__ void k_solve_bodies(DBodies B, DContacts C, int n) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    int b1 = C.b1[c], b2 = C.b2[c];
    C.sb1[c] = B.parent[b1] >= 0 ? B.parent[b1] : b1;
    C.sb2[c] = B.parent[b2] >= 0 ? B.parent[b2] : b2;
}

// MotionMetricProcessor.getLargestVelocityNorm (MotionMetricProcessor.java:39-73)
__device__ __forceinline__ v3 spatial_vel(const DBodies& B, int b, v3 pW) {
    v3 t = sub(pW, ldv(B.x + 3 * b));
    return add(cross(ldv(B.w + 3 * b), t), ldv(B.v + 3 * b));
}

__global__ void k_metrics(DBodies B, const int* pa, const int* pb, const int* mode, int n, const int* nbb,
                          double* out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int a = pa[k], b = pb[k], m = mode[k];
    double largest = 0;
    if (m == 1) {   // single body (the other one is pinned)
        m3 R = ldm(B.R + 9 * a);
        v3 x = ldv(B.x + 3 * a);
        for (int q = 0; q < nbb[a]; q++) {
            v3 pW = tpoint(R, x, ldv(B.bbB + 24 * a + 3 * q));
            largest = jmax(length(spatial_vel(B, a, pW)), largest);
        }
    } else {
        for (int i = 0; i < 2; i++) {
            int body = i == 0 ? a : b;
            m3 R = ldm(B.R + 9 * body);
            v3 x = ldv(B.x + 3 * body);
            for (int q = 0; q < nbb[body]; q++) {
                v3 pW = tpoint(R, x, ldv(B.bbB + 24 * body + 3 * q));
                v3 v1 = spatial_vel(B, a, pW), v2 = spatial_vel(B, b, pW);
                largest = jmax(length(sub(v1, v2)), largest);
            }
        }
    }
    out[k] = largest;
}

// ---------------------------------------------------------------------------
// host restatement of RigidCollection arithmetic on the host body mirror
namespace {

inline m3 getOp(const HostWorld& h, int b, v3 com) {   // RigidCollection.getOp (RigidCollection.java:809-830)
    double x = h.x[3 * b] - com.x, y = h.x[3 * b + 1] - com.y, z = h.x[3 * b + 2] - com.z;
    double x2 = x * x, y2 = y * y, z2 = z * z;
    m3 op;
    op.m[0] = y2 + z2; op.m[1] = -x * y; op.m[2] = -x * z;
    op.m[3] = -y * x; op.m[4] = x2 + z2; op.m[5] = -y * z;
    op.m[6] = -z * x; op.m[7] = -z * y; op.m[8] = x2 + y2;
    double m = h.mass[b];
    for (int k = 0; k < 9; k++) op.m[k] *= m;
    return op;
}
inline m3 madd(const m3& a, const m3& b) { m3 r; for (int k = 0; k < 9; k++) r.m[k] = a.m[k] + b.m[k]; return r; }
inline m3 msub(const m3& a, const m3& b) { m3 r; for (int k = 0; k < 9; k++) r.m[k] = a.m[k] - b.m[k]; return r; }
inline v3 X(const HostWorld& h, int b) { return ldv(&h.x[3 * b]); }
inline m3 Rm(const HostWorld& h, int b) { return ldm(&h.R[9 * b]); }
inline bool pinned(const HostWorld& h, int b) { return h.flags[b] & F_PINNED; }
inline bool sleeping(const HostWorld& h, int b) { return h.flags[b] & F_SLEEPING; }
inline void setSleeping(HostWorld& h, int b, bool s) { if (s) h.flags[b] |= F_SLEEPING; else h.flags[b] &= ~F_SLEEPING; }
inline void setPinned(HostWorld& h, int b, bool s) { if (s) h.flags[b] |= F_PINNED; else h.flags[b] &= ~F_PINNED; }
inline bool sameColl(const HostWorld& h, int a, int b) { return h.parent[a] >= 0 && h.parent[a] == h.parent[b]; }

// RigidTransform3D.multAinvB: R = A.R^T B.R, t = A.R^T (B.t - A.t)
inline void multAinvB(const m3& AR, v3 At, const m3& BR, v3 Bt, m3& R, v3& t) {
    m3 ART;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) ART.m[3 * i + j] = AR.m[3 * j + i];
    t = mxv(ART, sub(Bt, At));
    R = mmul(ART, BR);
}

}  // namespace

void HostMerge::reset(int cap) {
    bpc.clear();
    coll.clear();
    bodyBpcs.assign(cap, OSetI());
    index.clear();
    freeSlots.clear();
    nSlots = 0;
}

int HostMerge::findOrCreate(int a, int b) {
    uint64_t k = ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
    auto it = index.find(k);
    if (it != index.end() && coll.contains(it->second)) return it->second;
    for (int q : coll.v) {   // BodyPairContact.checkExists semantics when the index is stale
        const HBPC& p = bpc[q];
        if ((p.a == a && p.b == b) || (p.a == b && p.b == a)) { index[k] = q; return q; }
    }
    HBPC p;
    p.a = a;
    p.b = b;
    bpc.push_back(p);
    int id = (int)bpc.size() - 1;
    coll.add(id);
    index[k] = id;
    return id;
}

// ---------------------------------------------------------------------------
// Ctx: merging-enabled step
void Ctx::addToBodyLists(int p) { HBPC& q = M.bpc[p]; M.bodyBpcs[q.a].add(p); M.bodyBpcs[q.b].add(p); }
void Ctx::addToBodyListsParent(int p) {
    HBPC& q = M.bpc[p];
    if (host.parent[q.a] >= 0) M.bodyBpcs[host.parent[q.a]].add(p);
    if (host.parent[q.b] >= 0) M.bodyBpcs[host.parent[q.b]].add(p);
}
void Ctx::removeFromBodyLists(int p) { HBPC& q = M.bpc[p]; M.bodyBpcs[q.a].remove(p); M.bodyBpcs[q.b].remove(p); }
void Ctx::removeFromBodyListsParent(int p) {
    HBPC& q = M.bpc[p];
    if (host.parent[q.a] >= 0) M.bodyBpcs[host.parent[q.a]].remove(p);
    if (host.parent[q.b] >= 0) M.bodyBpcs[host.parent[q.b]].remove(p);
}

void Ctx::removeEmptyBodyPairContacts() {   // CollisionProcessor.java:182-200
    std::vector<int> keep;
    bool updated = false;
    for (int p : M.coll.v) {
        if (!M.bpc[p].list.empty()) keep.push_back(p);
        else { removeFromBodyLists(p); removeFromBodyListsParent(p); updated = true; }
    }
    if (updated) {
        M.coll.clear();
        for (int p : keep) M.coll.add(p);
    }
}

// CollisionProcessor.updateBodyPairContacts / storeInBodyPairContacts (:145-176)
int Ctx::updateBodyPairContacts() {
    keyB1.resize(nContacts);
    keyB2.resize(nContacts);
    if (nContacts) {
        cudaMemcpyAsync(keyB1.data(), C[cur].b1, sizeof(int) * nContacts, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(keyB2.data(), C[cur].b2, sizeof(int) * nContacts, cudaMemcpyDeviceToHost, stream);
        int r = syncErr();
        if (r) return r;
    }
    for (int p : M.coll.v) { M.bpc[p].checked = false; M.bpc[p].list.clear(); }
    for (int b : host.top)
        if (host.flags[b] & F_COLLECTION)
            for (int p : M.bodyBpcs[b].v) M.bpc[p].checked = false;
    for (int c = 0; c < nContacts; c++) {
        int a = keyB1[c], b = keyB2[c];
        if (pinned(host, a) && pinned(host, b)) continue;
        int p = M.findOrCreate(a, b);
        addToBodyLists(p);
        addToBodyListsParent(p);
        M.bpc[p].list.push_back(c);
    }
    removeEmptyBodyPairContacts();
    return AM_OK;
}

// download everything the host-side collection arithmetic reads
int Ctx::pullBodies() {
    HostWorld& h = host;
    int cap = h.cap;
    cudaMemcpyAsync(h.x.data(), B.x, sizeof(double) * 3 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.R.data(), B.R, sizeof(double) * 9 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.v.data(), B.v, sizeof(double) * 3 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.w.data(), B.w, sizeof(double) * 3 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.M.data(), B.M, sizeof(double) * 9 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.jinv.data(), B.jinv, sizeof(double) * 9 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(h.flags.data(), B.flags, sizeof(int) * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(devDv.data(), B.dv, sizeof(double) * 6 * cap, cudaMemcpyDeviceToHost, stream);
    return syncErr();
}

int Ctx::pushBodies() {
    HostWorld& h = host;
    int cap = h.cap;
    cudaMemcpyAsync(B.x, h.x.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.R, h.R.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.v, h.v.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.w, h.w.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.M, h.M.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.M0, h.M0.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.jinv, h.jinv.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.jinv0, h.jinv0.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.mass, h.mass.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.minv, h.minv.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.bbB, h.bbB.data(), sizeof(double) * 24 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.B2C, h.B2C.data(), sizeof(double) * 12 * cap, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(B.dv, devDv.data(), sizeof(double) * 6 * cap, cudaMemcpyHostToDevice, stream);
    std::vector<int> nbb(cap);
    for (int b = 0; b < cap; b++) nbb[b] = h.nbb[b];
    cudaMemcpyAsync(nbbDev, nbb.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream);
    return uploadTopology();
}

// ---- collection store of contacts ------------------------------------------
int Ctx::ensureStore(int need) {
    if (need <= I.cap) return AM_OK;
    int cap = std::max(need * 2, 4096);
    DContacts n;
    std::memset(&n, 0, sizeof(n));
    if (allocContacts(n, cap)) return AM_E_CUDA;
    if (I.cap > 0 && M.nSlots > 0) {   // carry the live slots over
        std::vector<int> idx(M.nSlots);
        for (int k = 0; k < M.nSlots; k++) idx[k] = k;
        int r = copyContacts(I, idx, n, idx, 0);
        if (r) return r;
    }
    I = n;
    return AM_OK;
}

int Ctx::copyContacts(const DContacts& S, const std::vector<int>& si, DContacts& D, const std::vector<int>& di,
                      int mode) {
    int n = (int)si.size();
    if (n == 0) return AM_OK;
    if (n > idxCap) {
        int cap = std::max(n * 2, 4096);
        if (alloc(&idxA, cap) || alloc(&idxB, cap)) return AM_E_CUDA;
        idxCap = cap;
    }
    cudaMemcpyAsync(idxA, si.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(idxB, di.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    k_copy_contacts<<<(n + 127) / 128, 128, 0, stream>>>(S, idxA, D, idxB, n, mode);
    AM_LAUNCHED(1);
    return syncErr();   // index buffers are reused by the next copy
}

int Ctx::newSlot() {
    if (!M.freeSlots.empty()) { int s = M.freeSlots.back(); M.freeSlots.pop_back(); return s; }
    return M.nSlots++;
}

// RigidCollection.addToInternalContact (RigidCollection.java:836-847)
int Ctx::toInternal(int p) {
    HBPC& q = M.bpc[p];
    std::vector<int> ext, extDst, in, inDst;
    std::vector<int> newList;
    for (int ref : q.list) {
        int s = newSlot();
        if (ref >= 0) { ext.push_back(ref); extDst.push_back(s); }
        else { in.push_back(~ref); inDst.push_back(s); }
        newList.push_back(~s);
    }
    int r = ensureStore(M.nSlots + 1);
    if (r) return r;
    if ((r = copyContacts(C[cur], ext, I, extDst, 1))) return r;
    if (!in.empty()) {
        // copy within the store: stage through the sweep buffer to avoid aliasing
        if ((r = ensureSweep((int)in.size()))) return r;
        std::vector<int> tmp(in.size());
        for (size_t k = 0; k < in.size(); k++) tmp[k] = (int)k;
        if ((r = copyContacts(I, in, Sw, tmp, 0))) return r;
        if ((r = copyContacts(Sw, tmp, I, inDst, 1))) return r;
        for (int s : in) M.freeSlots.push_back(s);
    }
    q.list = newList;
    return AM_OK;
}

int Ctx::ensureSweep(int need) {
    if (need <= Sw.cap) return AM_OK;
    DContacts n;
    std::memset(&n, 0, sizeof(n));
    if (allocContacts(n, std::max(need * 2, 4096))) return AM_E_CUDA;
    Sw = n;
    return AM_OK;
}

// ---- single sweep in collections (CollisionProcessor.updateInCollections,
//      getOrganizedContacts, getNextLayer: CollisionProcessor.java:232-441)
void Ctx::nextLayer(std::vector<int>& layer, std::vector<int>& ordered) {
    std::vector<int> next;
    for (int p : layer)
        for (int i = 0; i < 2; i++) {
            int body = i == 0 ? M.bpc[p].a : M.bpc[p].b;
            for (int o : M.bodyBpcs[body].v)
                if (!M.bpc[o].checked) { next.push_back(o); M.bpc[o].checked = true; }
        }
    if (!next.empty()) {
        for (int p : next) ordered.push_back(p);
        nextLayer(next, ordered);
    }
}

// CollisionProcessor.getOrganizedContacts (:337-364) with getNextLayer: the
// pairs touching a fresh contact first, then breadth-first layers of their
// neighbours, then the remaining pairs of the collision list and of awake
// collections; the contacts of each pair in list order.  refs >= 0 index the
// current contact list, refs < 0 are ~slot of a contact inside a collection.
int Ctx::singleSweepOrder(std::vector<int>& refs) {
    refs.clear();
    // the same flags updateBodyPairContacts clears, so the order can be asked for again
    for (int p : M.coll.v) M.bpc[p].checked = false;
    for (int b : host.top)
        if (host.flags[b] & F_COLLECTION)
            for (int p : M.bodyBpcs[b].v) M.bpc[p].checked = false;
    // fresh flags of this step's contacts (set by the warm start)
    freshH.resize(nContacts);
    if (nContacts) {
        cudaMemcpyAsync(freshH.data(), C[cur].fresh, sizeof(int) * nContacts, cudaMemcpyDeviceToHost, stream);
        int r = syncErr();
        if (r) return r;
    }
    const double tOrder = phaseNow();   // CollisionProcessor.java:256-258 contactOrderingTime
    std::vector<int> ordered;
    for (int p : M.coll.v)
        for (int ref : M.bpc[p].list)
            if (ref >= 0 && freshH[ref]) { ordered.push_back(p); M.bpc[p].checked = true; break; }
    if (!ordered.empty()) {
        std::vector<int> first = ordered;
        nextLayer(first, ordered);
    }
    for (int p : M.coll.v)
        if (!M.bpc[p].checked) { ordered.push_back(p); M.bpc[p].checked = true; }
    for (int b : host.top)
        if ((host.flags[b] & F_COLLECTION) && !(host.flags[b] & F_SLEEPING))
            for (int p : M.bodyBpcs[b].v)
                if (!M.bpc[p].checked) { ordered.push_back(p); M.bpc[p].checked = true; }
    phaseAdd(AM_PHASE_CONTACT_ORDERING, tOrder);
    for (int p : ordered)
        for (int ref : M.bpc[p].list) refs.push_back(ref);
    return AM_OK;
}

// The single sweep of CollisionProcessor.updateInCollections (:262-302) over
// `refs` in the given order: Jacobians of contacts on collection members
// recomputed, b and D in collection mode, Gauss-Seidel in list order
// (iterations_in_collection passes), results scattered back; then the
// collections' sub-body velocities (RigidCollection.java:866-937).
int Ctx::singleSweepRefs(const std::vector<int>& refs, double dt) {
    std::vector<int> ext, extPos, in, inPos;
    int n = 0;
    for (int ref : refs) {
        if (ref >= 0) {
            if (ref >= nContacts) { err = "single sweep: contact index out of range"; return AM_E_ARG; }
            ext.push_back(ref); extPos.push_back(n);
        } else {
            if (~ref >= M.nSlots) { err = "single sweep: collection contact slot out of range"; return AM_E_ARG; }
            in.push_back(~ref); inPos.push_back(n);
        }
        n++;
    }
    int r = ensureSweep(n);
    if (r) return r;
    if ((r = copyContacts(C[cur], ext, Sw, extPos, 0))) return r;
    if ((r = copyContacts(I, in, Sw, inPos, 0))) return r;
    if (n > 0) {
        k_recompute_J<<<(n + 127) / 128, 128, 0, stream>>>(B, Sw, n, 1);
        AM_LAUNCHED(1);
        launch_solve_prep(B, Sw, n, dt, P.feedback_stiffness, true, P.restitution_override, P.restitution, 0, stream);
        const double tPgs = phaseNow();   // CollisionProcessor.java:284-287 singleItPGSTime
        if ((r = exactSweep(Sw, n, P.iterations_in_collection, true))) return r;
        phaseAdd(AM_PHASE_SINGLE_IT_PGS, tPgs);
        if ((r = copyContacts(Sw, extPos, C[cur], ext, 2))) return r;
        if ((r = copyContacts(Sw, inPos, I, in, 2))) return r;
    }
    launch_sub_adv_vel(B, top, ntop, subOff, subIds, dt, stream);
    return syncErr();
}

bool Ctx::anyCollection() const {
    for (int b : host.top) if (host.flags[b] & F_COLLECTION) return true;
    return false;
}

int Ctx::singleSweep(double dt) {
    if (!P.update_contacts_in_collections || !anyCollection()) return AM_OK;
    std::vector<int> refs;
    int r = singleSweepOrder(refs);
    return r ? r : singleSweepRefs(refs, dt);
}

// ---- motion metrics on the device ------------------------------------------
int Ctx::metrics(const std::vector<int>& a, const std::vector<int>& b, const std::vector<int>& mode,
                 std::vector<double>& out) {
    int n = (int)a.size();
    out.assign(n, 0.0);
    if (n == 0) return AM_OK;
    if (n > metCap) {
        int cap = std::max(2 * n, 1024);
        if (alloc(&metA, cap) || alloc(&metB, cap) || alloc(&metM, cap) || alloc(&metOut, cap)) return AM_E_CUDA;
        metCap = cap;
    }
    cudaMemcpyAsync(metA, a.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(metB, b.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(metM, mode.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    k_metrics<<<(n + 127) / 128, 128, 0, stream>>>(B, metA, metB, metM, n, nbbDev, metOut);
    AM_LAUNCHED(1);
    cudaMemcpyAsync(out.data(), metOut, sizeof(double) * n, cudaMemcpyDeviceToHost, stream);
    return syncErr();
}

// BodyPairContact.accumulateForUnmerging (BodyPairContact.java:127-145) for
// every awake collection (RigidBodySystem.java:325-335)
int Ctx::accumulateForUnmerging() {
    std::vector<int> ids, a, b, mode;
    for (int t : host.top) {
        if (!(host.flags[t] & F_COLLECTION) || sleeping(host, t)) continue;
        for (int p : M.bodyBpcs[t].v) {
            HBPC& q = M.bpc[p];
            if (!sameColl(host, q.a, q.b)) continue;
            ids.push_back(p);
            if (pinned(host, q.a)) { a.push_back(q.b); b.push_back(q.b); mode.push_back(1); }
            else if (pinned(host, q.b)) { a.push_back(q.a); b.push_back(q.a); mode.push_back(1); }
            else { a.push_back(q.a); b.push_back(q.b); mode.push_back(2); }
        }
    }
    std::vector<double> m;
    int r = metrics(a, b, mode, m);
    if (r) return r;
    for (size_t k = 0; k < ids.size(); k++) {
        HBPC& q = M.bpc[ids[k]];
        if (m[k] > P.threshold_unmerge) q.mm.push_back(m[k]);
        else q.mm.clear();
    }
    return AM_OK;
}

// contact states of every contact a body-pair list refers to
int Ctx::pullStates(bool internalToo) {
    stateH.resize(nContacts);
    lam0H.resize(nContacts);
    cvH.resize(2 * (size_t)nContacts);
    if (nContacts) {
        cudaMemcpyAsync(stateH.data(), C[cur].state, sizeof(int) * nContacts, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(lam0H.data(), C[cur].lam, sizeof(double) * nContacts, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(cvH.data(), C[cur].cv, sizeof(double) * nContacts, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(cvH.data() + nContacts, C[cur].pcv, sizeof(double) * nContacts, cudaMemcpyDeviceToHost, stream);
    }
    if (internalToo && M.nSlots) {
        istateH.resize(M.nSlots);
        cudaMemcpyAsync(istateH.data(), I.state, sizeof(int) * M.nSlots, cudaMemcpyDeviceToHost, stream);
    }
    return syncErr();
}

// ---- RigidCollection operations on the host mirror --------------------------
int Ctx::newCollectionSlot() {
    HostWorld& h = host;
    for (int b = h.n; b < h.cap; b++)
        if (h.type[b] == -1 && !(h.flags[b] & F_COLLECTION)) return b;
    return -1;
}

void Ctx::collApplyVelocitiesTo(int c, int b) {   // RigidCollection.applyVelocitiesTo (:925-937)
    HostWorld& h = host;
    v3 r = sub(X(h, b), X(h, c));
    v3 wxr = cross(ldv(&h.w[3 * c]), r);
    stv(&h.v[3 * b], add(ldv(&h.v[3 * c]), wxr));
    stv(&h.w[3 * b], ldv(&h.w[3 * c]));
}

void Ctx::collUpdateState(int c, int b) {         // updateCollectionState (:459-469)
    HostWorld& h = host;
    setPinned(h, c, pinned(h, c) || pinned(h, b));
    setSleeping(h, c, sleeping(h, c) || sleeping(h, b));
    setSleeping(h, b, false);
}

void Ctx::collUpdateBB(int c, int b) {            // updateBB(RigidBody) (:637-668)
    HostWorld& h = host;
    if (h.nbb[c] == 0) return;
    if (h.type[b] == AM_PLANE) return;
    v3 mx = mk(-1.79769313486231570e308, -1.79769313486231570e308, -1.79769313486231570e308);
    v3 mn = mk(1.79769313486231570e308, 1.79769313486231570e308, 1.79769313486231570e308);
    for (int i = 0; i < 2; i++) {
        int q = i == 0 ? c : b;
        for (int k = 0; k < h.nbb[q]; k++) {
            v3 p = tpoint(Rm(h, q), X(h, q), ldv(&h.bbB[24 * q + 3 * k]));
            mn.x = std::min(mn.x, p.x); mn.y = std::min(mn.y, p.y); mn.z = std::min(mn.z, p.z);
            mx.x = std::max(mx.x, p.x); mx.y = std::max(mx.y, p.y); mx.z = std::max(mx.z, p.z);
        }
    }
    setBB(c, mn, mx);
}

void Ctx::setBB(int c, v3 mn, v3 mx) {
    double* bb = &host.bbB[24 * c];
    stv(bb + 12, mn);
    stv(bb + 15, mk(mn.x, mx.y, mx.z));
    stv(bb + 18, mk(mx.x, mn.y, mx.z));
    stv(bb + 21, mk(mx.x, mx.y, mn.z));
    stv(bb + 0, mx);
    stv(bb + 3, mk(mx.x, mn.y, mn.z));
    stv(bb + 6, mk(mn.x, mx.y, mn.z));
    stv(bb + 9, mk(mn.x, mn.y, mx.z));
}

void Ctx::collUpdateBBAll(int c) {                // updateBB() (:601-631)
    HostWorld& h = host;
    if (h.nbb[c] == 0) return;
    v3 mx = mk(-1.79769313486231570e308, -1.79769313486231570e308, -1.79769313486231570e308);
    v3 mn = mk(1.79769313486231570e308, 1.79769313486231570e308, 1.79769313486231570e308);
    for (int b : h.subs[c]) {
        if (h.type[b] == AM_PLANE) continue;
        m3 R = ldm(&h.B2C[12 * b]);
        v3 t = ldv(&h.B2C[12 * b + 9]);
        for (int k = 0; k < h.nbb[b]; k++) {
            v3 p = tpoint(R, t, ldv(&h.bbB[24 * b + 3 * k]));
            mn.x = std::min(mn.x, p.x); mn.y = std::min(mn.y, p.y); mn.z = std::min(mn.z, p.z);
            mx.x = std::max(mx.x, p.x); mx.y = std::max(mx.y, p.y); mx.z = std::max(mx.z, p.z);
        }
    }
    setBB(c, mn, mx);
}

void Ctx::collAddInternal(int c, int b) {          // addBodyInternalMethod (:477-514)
    HostWorld& h = host;
    m3 tR = Rm(h, c);
    v3 tt = X(h, c);
    stm(&h.R[9 * c], ident());                     // updateTheta
    if (pinned(h, c)) {
        stv(&h.v[3 * c], mk(0, 0, 0)); stv(&h.w[3 * c], mk(0, 0, 0));
        stm(&h.M[9 * c], zero3()); stm(&h.M0[9 * c], zero3()); stm(&h.jinv[9 * c], zero3()); stm(&h.jinv0[9 * c], zero3());
        h.mass[c] = 0; h.minv[c] = 0;
    } else {
        v3 com = X(h, c);
        double mc = h.mass[c], mb = h.mass[b];
        com.x *= mc; com.y *= mc; com.z *= mc;
        com = scaleadd(mb, X(h, b), com);
        double tmi = 1. / (mb + mc);
        com.x *= tmi; com.y *= tmi; com.z *= tmi;
        v3 v = ldv(&h.v[3 * c]);
        v.x *= mc; v.y *= mc; v.z *= mc;
        v = scaleadd(mb, ldv(&h.v[3 * b]), v);
        v.x *= tmi; v.y *= tmi; v.z *= tmi;
        stv(&h.v[3 * c], v);
        v3 w = ldv(&h.w[3 * c]);
        w.x *= mc; w.y *= mc; w.z *= mc;
        w = scaleadd(mb, ldv(&h.w[3 * b]), w);
        w.x *= tmi; w.y *= tmi; w.z *= tmi;
        stv(&h.w[3 * c], w);
        m3 m0 = zero3();                           // updateInertia (:779-790)
        for (int i = 0; i < 2; i++) {
            int q = i == 0 ? c : b;
            m0 = madd(m0, ldm(&h.M[9 * q]));
            m0 = madd(m0, getOp(h, q, com));
        }
        stm(&h.M[9 * c], m0);
        collUpdateBB(c, b);
        h.mass[c] = mc + mb;
        h.minv[c] = tmi;
        stv(&h.x[3 * c], com);
        for (int k = 0; k < h.nbb[c]; k++) {
            v3 p = tinvpoint(Rm(h, c), X(h, c), ldv(&h.bbB[24 * c + 3 * k]));
            stv(&h.bbB[24 * c + 3 * k], p);
        }
    }
    m3 R;
    v3 t;
    multAinvB(Rm(h, c), X(h, c), tR, tt, R, t);
    stm(&h.B2C[12 * c], R);
    stv(&h.B2C[12 * c + 9], t);
}

void Ctx::collInertiaRestInvert(int c) {           // updateInertiaRestAndInvert (:674-680)
    HostWorld& h = host;
    if (pinned(h, c)) return;
    m3 Mw = ldm(&h.M[9 * c]), Ji;
    if (!invert3(Mw, Ji)) Ji = zero3();
    stm(&h.jinv[9 * c], Ji);
    stm(&h.M0[9 * c], rtmr(Rm(h, c), Mw));
    stm(&h.jinv0[9 * c], rtmr(Rm(h, c), Ji));
}

void Ctx::rotInertia(int b) {                      // RigidBody.updateRotationalInertiaFromTransformation
    HostWorld& h = host;
    if (pinned(h, b)) return;
    stm(&h.M[9 * b], rm0rt(Rm(h, b), ldm(&h.M0[9 * b])));
    stm(&h.jinv[9 * b], rm0rt(Rm(h, b), ldm(&h.jinv0[9 * b])));
}

void Ctx::collBodiesTransforms(int c) {            // updateBodiesTransformations (:588-591)
    HostWorld& h = host;
    for (int b : h.subs[c]) {
        m3 R;
        v3 t;
        multAinvB(Rm(h, c), X(h, c), Rm(h, b), X(h, b), R, t);
        stm(&h.B2C[12 * b], R);
        stv(&h.B2C[12 * b + 9], t);
    }
}

void Ctx::collAddBody(int c, int b) {              // addBody (:128-139)
    host.parent[b] = c;
    host.subs[c].push_back(b);
    collUpdateState(c, b);
    collAddInternal(c, b);
    collInertiaRestInvert(c);
    rotInertia(c);
    collBodiesTransforms(c);
}

void Ctx::collAddBodies(int c, const std::vector<int>& bs) {   // addBodies (:145-158)
    for (int b : bs) {
        host.parent[b] = c;
        host.subs[c].push_back(b);
        collUpdateState(c, b);
        collAddInternal(c, b);
    }
    collInertiaRestInvert(c);
    rotInertia(c);
    collBodiesTransforms(c);
}

void Ctx::collAddCollection(int c, int o) {        // addCollection (:164-178)
    for (int b : host.subs[o]) { host.parent[b] = c; host.subs[c].push_back(b); }
    collUpdateState(c, o);
    collAddInternal(c, o);
    collInertiaRestInvert(c);
    rotInertia(c);
    collBodiesTransforms(c);
}

void Ctx::freeCollection(int c) {
    HostWorld& h = host;
    h.subs[c].clear();
    h.flags[c] = 0;
    h.type[c] = -1;
    h.parent[c] = -1;
    M.bodyBpcs[c].clear();
}

int Ctx::newCollection(int b1, int b2) {           // RigidCollection(body1, body2) (:55-76)
    HostWorld& h = host;
    int c = newCollectionSlot();
    if (c < 0) return -1;
    h.type[c] = -1;
    h.flags[c] = F_COLLECTION;
    h.parent[c] = -1;
    h.subs[c].clear();
    M.bodyBpcs[c].clear();
    h.friction[c] = 0.8;
    h.restitution[c] = 0;
    for (int k = 0; k < 12; k++) h.B2C[12 * c + k] = 0.0;
    for (int k = 0; k < 6; k++) devDv[6 * c + k] = 0.0;
    auto setFrom = [&](int b) {                     // RigidBody.set (RigidBody.java:248-271)
        for (int k = 0; k < 3; k++) { h.v[3 * c + k] = h.v[3 * b + k]; h.w[3 * c + k] = h.w[3 * b + k]; h.x[3 * c + k] = h.x[3 * b + k]; }
        for (int k = 0; k < 9; k++) {
            h.R[9 * c + k] = h.R[9 * b + k]; h.M[9 * c + k] = h.M[9 * b + k]; h.M0[9 * c + k] = h.M0[9 * b + k];
            h.jinv[9 * c + k] = h.jinv[9 * b + k]; h.jinv0[9 * c + k] = h.jinv0[9 * b + k];
        }
        h.mass[c] = h.mass[b]; h.minv[c] = h.minv[b];
        setPinned(h, c, pinned(h, b));
        setSleeping(h, c, sleeping(h, b));
        h.nbb[c] = h.nbb[b];
        for (int k = 0; k < 24; k++) h.bbB[24 * c + k] = h.bbB[24 * b + k];
    };
    if (h.type[b1] == AM_PLANE) {
        setFrom(b2);
        h.parent[b2] = c;
        h.subs[c].push_back(b2);
        collAddBody(c, b1);
    } else {
        setFrom(b1);
        h.parent[b1] = c;
        h.subs[c].push_back(b1);
        collAddBody(c, b2);
    }
    return c;
}

void Ctx::collRemoveBodies(int c, const std::vector<int>& rm) {   // removeBodies (:686-753)
    HostWorld& h = host;
    std::vector<int> keep;
    for (int b : h.subs[c])
        if (std::find(rm.begin(), rm.end(), b) == rm.end()) keep.push_back(b);
    h.subs[c] = keep;
    m3 tR = Rm(h, c);
    v3 tt = X(h, c);
    bool wasPinned = pinned(h, c);
    bool pin = false;
    for (int b : h.subs[c]) pin = pin || pinned(h, b);
    setPinned(h, c, pin);
    stm(&h.R[9 * c], ident());
    if (pin) {
        stv(&h.v[3 * c], mk(0, 0, 0)); stv(&h.w[3 * c], mk(0, 0, 0));
        stm(&h.M[9 * c], zero3()); stm(&h.M0[9 * c], zero3()); stm(&h.jinv[9 * c], zero3()); stm(&h.jinv0[9 * c], zero3());
        h.mass[c] = 0; h.minv[c] = 0;
    } else if (wasPinned) {
        v3 x = mk(0, 0, 0);
        double m = 0;
        for (int b : h.subs[c]) { x = scaleadd(h.mass[b], X(h, b), x); m += h.mass[b]; }
        h.mass[c] = m;
        h.minv[c] = 1. / m;
        x.x *= h.minv[c]; x.y *= h.minv[c]; x.z *= h.minv[c];
        stv(&h.x[3 * c], x);
        m3 Mw = zero3();                            // computeInertia (:764-772)
        for (int b : h.subs[c]) { Mw = madd(Mw, ldm(&h.M[9 * b])); Mw = madd(Mw, getOp(h, b, x)); }
        stm(&h.M[9 * c], Mw);
        collInertiaRestInvert(c);
    } else {
        for (int b : rm) {
            v3 com = X(h, c);
            double mc = h.mass[c];
            com.x *= mc; com.y *= mc; com.z *= mc;
            v3 x = scaleadd(-h.mass[b], X(h, b), com);
            double inv = 1. / mc;
            com.x *= inv; com.y *= inv; com.z *= inv;
            h.mass[c] = mc - h.mass[b];
            h.minv[c] = 1. / h.mass[c];
            x.x *= h.minv[c]; x.y *= h.minv[c]; x.z *= h.minv[c];
            stv(&h.x[3 * c], x);
            m3 Mw = msub(ldm(&h.M[9 * c]), ldm(&h.M[9 * b]));   // updateInertiaReverse (:797-806)
            for (int i = 0; i < 2; i++) {
                int q = i == 0 ? c : b;
                Mw = msub(Mw, getOp(h, q, com));
            }
            stm(&h.M[9 * c], Mw);
        }
        collInertiaRestInvert(c);
    }
    rotInertia(c);
    collBodiesTransforms(c);
    collUpdateBBAll(c);
    m3 R;
    v3 t;
    multAinvB(Rm(h, c), X(h, c), tR, tt, R, t);
    stm(&h.B2C[12 * c], R);
    stv(&h.B2C[12 * c + 9], t);
}

void Ctx::collAddBPCs(int p) {                     // addBPCsToCollection (:854-863)
    addToBodyListsParent(p);
    for (int i = 0; i < 2; i++) {
        int b = i == 0 ? M.bpc[p].a : M.bpc[p].b;
        std::vector<int> snap = M.bodyBpcs[b].v;
        for (int e : snap) addToBodyListsParent(e);
    }
}

void Ctx::collFillInternal(int c) {                // fillInternalBodyContacts (:959-978)
    M.bodyBpcs[c].clear();
    for (int b : host.subs[c])
        for (int p : M.bodyBpcs[b].v)
            if (!M.bodyBpcs[c].contains(p)) {
                M.bodyBpcs[c].add(p);
                int o = M.bpc[p].a == b ? M.bpc[p].b : M.bpc[p].a;
                if (sameColl(host, b, o)) M.bpc[p].inCollection = true;
            }
}

int Ctx::collAddIncomplete(int body, std::vector<int>& removal) {   // addIncompleteContacts (:987-998)
    std::vector<int> snap = M.bodyBpcs[body].v;
    for (int p : snap) {
        HBPC& q = M.bpc[p];
        if (sameColl(host, q.a, q.b) && !q.inCollection) {
            q.inCollection = true;
            q.mm.clear();
            q.sh.clear();
            int r = toInternal(p);
            if (r) return r;
            collAddBPCs(p);
            removal.push_back(p);
        }
    }
    return AM_OK;
}

void Ctx::collUnmergeBody(int c, int b) {          // unmergeBody (:944-953)
    collApplyVelocitiesTo(c, b);
    for (int k = 0; k < 6; k++) devDv[6 * b + k] = 0.0;
    host.parent[b] = -1;
}

// ---- Merging.merge (Merging.java:73-163) -------------------------------------
static void listRemove(std::vector<int>& v, int b) {
    for (size_t i = 0; i < v.size(); i++) if (v[i] == b) { v.erase(v.begin() + i); return; }
}

bool Ctx::checkMergeCondition(int p) {             // BodyPairContact.java:151-224
    HBPC& q = M.bpc[p];
    // A body with a prescribed motion (am_set_kinematic) never merges: a
    // collection that holds a pinned body stays put, so the motion would stop
    // acting on the body's contacts while it moved through the members merged
    // with it.  The reference's pinned bodies never move; this is the only
    // addition to its test.
    for (const Kinematic& k : kin)
        if (k.body == q.a || k.body == q.b) return false;
    if (sleeping(host, q.a) && sleeping(host, q.b)) return true;
    if (P.enable_merge_let_it_breathe)
        for (int ref : q.list) {
            double cv, pcv;
            if (ref >= 0) { cv = cvH[ref]; pcv = cvH[nContacts + ref]; }
            else continue;   // pairs in the collision list hold current-step contacts only
            if (std::fabs(pcv - cv) > P.threshold_breath) return false;
        }
    if (!P.enable_merge_pinned && (pinned(host, q.a) || pinned(host, q.b))) return false;
    if (sameColl(host, q.a, q.b)) return false;
    if ((int)q.mm.size() == P.step_accum_merging) {
        for (double m : q.mm) if (m > P.threshold_merge) return false;
    } else return false;
    if (P.enable_merge_stable_contact) {
        if ((int)q.sh.size() == P.step_accum_merging) {
            for (int s : q.sh) if (s == AM_STATE_ONEDGE) return false;
        } else return false;
    }
    return true;
}

// The merge and unmerge predicates on the current state, read only: the
// pairs of the collision list in Merging.merge's order with
// checkMergeCondition (BodyPairContact.java:151-177), then the pairs inside
// every awake collection in Merging.unmerge's order with its selection test
// (checkContactsState or the relative-motion history, Merging.java:222-240).
// Sleeping bits are read from the device first (the step's sleep phase sets
// them there).
int Ctx::mergeTests(std::vector<int>& a, std::vector<int>& b, std::vector<int>& kind, std::vector<int>& result,
                    std::vector<double>& metric) {
    a.clear(); b.clear(); kind.clear(); result.clear(); metric.clear();
    if (!host.cap) { err = "no scene loaded"; return AM_E_STATE; }
    if (nScenes > 0) { err = "merging is not part of the batched step"; return AM_E_STATE; }
    cudaMemcpyAsync(host.flags.data(), B.flags, sizeof(int) * host.cap, cudaMemcpyDeviceToHost, stream);
    int r = pullStates(true);
    if (r) return r;
    auto put = [&](const HBPC& q, int k, bool res) {
        a.push_back(q.a);
        b.push_back(q.b);
        kind.push_back(k);
        result.push_back(res ? 1 : 0);
        metric.push_back(q.mm.empty() ? 0.0 : q.mm.back());
    };
    for (int p : M.coll.v) {
        if (M.bpc[p].inCollection) continue;
        put(M.bpc[p], 0, checkMergeCondition(p));
    }
    for (int t : host.top) {
        if (sleeping(host, t) || !(host.flags[t] & F_COLLECTION)) continue;
        for (int p : M.bodyBpcs[t].v) {
            const HBPC& q = M.bpc[p];
            if (!q.inCollection) continue;
            bool sel = false;
            for (int ref : q.list) {
                int st = ref >= 0 ? stateH[ref] : istateH[~ref];
                if ((st == AM_STATE_BROKEN && P.enable_unmerge_normal) ||
                    (st == AM_STATE_ONEDGE && P.enable_unmerge_friction)) { sel = true; break; }
            }
            if (!sel) sel = (int)q.mm.size() >= P.step_accum_unmerging && q.list.size() < 3;
            put(q, 1, sel);
        }
    }
    return AM_OK;
}

int Ctx::merge() {
    if (!P.enable_merging) return AM_OK;
    // condition inputs: violations of every contact the external pairs refer to
    int r = pullStates(false);
    if (r) return r;
    icvH.clear(); ipcvH.clear();
    bool pulled = false;
    std::vector<int> removal;
    std::vector<int> snapshot = M.coll.v;
    for (int p : snapshot) {
        if (M.bpc[p].inCollection || !checkMergeCondition(p)) continue;
        if (!pulled) { if ((r = pullBodies())) return r; pulled = true; }
        mergingEvent = true;
        mergeEvents++;
        HBPC& q = M.bpc[p];
        q.inCollection = true;
        q.mm.clear();
        q.sh.clear();
        removal.push_back(p);
        const double tb = phaseNow();   // Merging.java:80-155 mergingBuildTime
        int b1 = q.a, b2 = q.b;
        int p1 = host.parent[b1], p2 = host.parent[b2];
        if (p1 < 0 && p2 < 0) {
            listRemove(host.top, b1);
            listRemove(host.top, b2);
            int c = newCollection(b1, b2);
            if (c < 0) { err = "no free collection slot"; return AM_E_CAPACITY; }
            if ((r = toInternal(p))) return r;
            collAddBPCs(p);
            host.top.push_back(c);
        } else if (p1 >= 0 && p2 >= 0) {
            int big = p1, small = p2;
            if (!(host.subs[p1].size() > host.subs[p2].size())) { big = p2; small = p1; }
            listRemove(host.top, small);
            for (int e : M.bodyBpcs[small].v) M.bodyBpcs[big].add(e);
            collAddCollection(big, small);
            freeCollection(small);
            if ((r = toInternal(p))) return r;
            std::vector<int> all = host.subs[big];
            for (int b : all) if ((r = collAddIncomplete(b, removal))) return r;
            collAddBPCs(p);
        } else if (p1 >= 0) {
            listRemove(host.top, b2);
            collAddBody(p1, b2);
            if ((r = toInternal(p))) return r;
            if ((r = collAddIncomplete(b2, removal))) return r;
            collAddBPCs(p);
        } else {
            listRemove(host.top, b1);
            collAddBody(p2, b1);
            if ((r = toInternal(p))) return r;
            if ((r = collAddIncomplete(b1, removal))) return r;
            collAddBPCs(p);
        }
        phaseAdd(AM_PHASE_MERGING_BUILD, tb);
    }
    for (int p : removal) M.coll.remove(p);
    if (pulled) return pushBodies();
    return AM_OK;
}

// ---- Merging.unmerge / unmergeSelectedBpcs / buildNeighborBody (Merging.java:215-393)
void Ctx::buildNeighbor(int b, OSetI& sub, OSetI& handled) {
    for (int p : M.bodyBpcs[b].v) {
        if (!M.bpc[p].inCollection) continue;
        int o = M.bpc[p].a == b ? M.bpc[p].b : (M.bpc[p].b == b ? M.bpc[p].a : -1);
        if (o < 0) continue;
        if (!sub.contains(o) && !handled.contains(o)) {
            sub.add(o);
            buildNeighbor(o, sub, handled);
        }
    }
}

int Ctx::unmergeSelected(int coll, OSetI& sel, std::vector<int>& newBodies, bool& removeCollection) {
    removeCollection = true;
    for (int p : sel.v) M.bpc[p].inCollection = false;
    OSetI handled, sub, remained;
    std::vector<int> snapshot = host.subs[coll];
    size_t ncoll = host.subs[coll].size();
    for (int b : snapshot) {
        if (handled.contains(b)) continue;
        sub.add(b);
        buildNeighbor(b, sub, handled);
        for (int q : sub.v) handled.add(q);
        if (ncoll != sub.size()) {
            if (sub.size() < ncoll / 2 + 1) {
                for (int q : sub.v) collUnmergeBody(coll, q);
                if (sub.size() > 1) {
                    int sb1 = sub.v[0], sb2 = sub.v[1];
                    std::vector<int> rest(sub.v.begin() + 2, sub.v.end());
                    int nc = newCollection(sb1, sb2);
                    if (nc < 0) { err = "no free collection slot"; return AM_E_CAPACITY; }
                    collAddBodies(nc, rest);
                    collFillInternal(nc);
                    newBodies.push_back(nc);
                } else if (sub.size() == 1) {
                    newBodies.push_back(sub.v[0]);
                }
            } else {
                removeCollection = false;
                for (int q : sub.v) remained.add(q);
            }
        } else {
            removeCollection = false;
            for (int q : sub.v) remained.add(q);
            break;
        }
        sub.clear();
    }
    // reconnect or hand back to the collision processor
    for (int p : sel.v) {
        HBPC& q = M.bpc[p];
        if (sameColl(host, q.a, q.b)) {
            q.inCollection = true;
        } else {
            if (!M.coll.contains(p)) {
                M.coll.add(p);
                // contacts re-enter CollisionProcessor.contacts with lambdaXwarm = lambdaX:
                // append copies to the current buffer and point the pair at them
                std::vector<int> slots, newIdx, newList;
                for (int ref : q.list) if (ref < 0) slots.push_back(~ref);
                int r = appendFromStore(slots, newIdx);
                if (r) return r;
                size_t k = 0;
                for (int ref : q.list) newList.push_back(ref >= 0 ? ref : newIdx[k++]);
                if (!newIdx.empty()) {
                    apA.push_back(q.a); apB.push_back(q.b);
                    apOff.push_back(newIdx.front()); apCnt.push_back((int)newIdx.size());
                }
                q.list = newList;
            }
            q.mm.clear();
            q.sh.clear();
        }
    }
    if (!removeCollection) {
        if (remained.size() != host.subs[coll].size()) {
            std::vector<int> rm;
            for (int q : handled.v) if (!remained.contains(q)) rm.push_back(q);
            collRemoveBodies(coll, rm);
            collFillInternal(coll);
        }
    }
    return AM_OK;
}

int Ctx::unmerge() {
    if (!P.enable_unmerging) return AM_OK;
    if (!P.enable_unmerge_relative_motion && !P.enable_unmerge_normal && !P.enable_unmerge_friction) return AM_OK;
    bool anyColl = false;
    for (int t : host.top) if (host.flags[t] & F_COLLECTION) anyColl = true;
    if (!anyColl) return AM_OK;
    int r = pullStates(true);
    if (r) return r;
    std::vector<int> removalQ, additionQ;
    std::vector<int> snapshot = host.top;
    bool pulled = false;
    for (int b : snapshot) {
        if (sleeping(host, b) || !(host.flags[b] & F_COLLECTION)) continue;
        OSetI sel;
        for (int p : M.bodyBpcs[b].v) {
            HBPC& q = M.bpc[p];
            if (!q.inCollection || sel.contains(p)) continue;
            bool state = false;   // BodyPairContact.checkContactsState (:255-266)
            for (int ref : q.list) {
                int st = ref >= 0 ? stateH[ref] : istateH[~ref];
                if (st == AM_STATE_BROKEN && P.enable_unmerge_normal) { state = true; break; }
                if (st == AM_STATE_ONEDGE && P.enable_unmerge_friction) { state = true; break; }
            }
            bool motion = (int)q.mm.size() >= P.step_accum_unmerging && q.list.size() < 3;
            if (!state && !motion) continue;
            sel.add(p);
        }
        if (sel.empty()) continue;
        if (!pulled) { if ((r = pullBodies())) return r; pulled = true; }
        const double tb = phaseNow();   // Merging.java:219-265 unmergingBuildTime
        std::vector<int> nb;
        bool removeC = false;
        if ((r = unmergeSelected(b, sel, nb, removeC))) return r;
        if (!nb.empty()) {
            mergingEvent = true;
            unmergeEvents++;
            for (int q : nb) additionQ.push_back(q);
            if (removeC) removalQ.push_back(b);
        }
        phaseAdd(AM_PHASE_UNMERGING_BUILD, tb);
    }
    for (int q : additionQ) host.top.push_back(q);
    if (!removalQ.empty()) {
        std::vector<int> keep;
        for (int q : host.top)
            if (std::find(removalQ.begin(), removalQ.end(), q) == removalQ.end()) keep.push_back(q);
        host.top = keep;
        for (int q : removalQ) freeCollection(q);
    }
    if (pulled) return pushBodies();
    return AM_OK;
}

// ---- clearBodyPairContacts + accumulateForMerging -----------------------------
int Ctx::clearBodyPairContacts() {                 // CollisionProcessor.java:213-226
    int r = pullStates(false);
    if (r) return r;
    for (int p : M.coll.v) {
        std::vector<int> keep;
        for (int ref : M.bpc[p].list)
            if (ref >= 0 && std::fabs(lam0H[ref]) > 1e-14) keep.push_back(ref);
        M.bpc[p].list = keep;
    }
    removeEmptyBodyPairContacts();
    return AM_OK;
}

int Ctx::accumulateForMerging() {                  // BodyPairContact.accumulateForMerging (:83-121)
    std::vector<int> a, b, mode;
    for (int p : M.coll.v) {
        HBPC& q = M.bpc[p];
        int b1 = host.parent[q.a] >= 0 ? host.parent[q.a] : q.a;
        int b2 = host.parent[q.b] >= 0 ? host.parent[q.b] : q.b;
        if (pinned(host, b1)) { a.push_back(b2); b.push_back(b2); mode.push_back(1); }
        else if (pinned(host, b2)) { a.push_back(b1); b.push_back(b1); mode.push_back(1); }
        else { a.push_back(b1); b.push_back(b2); mode.push_back(2); }
    }
    std::vector<double> m;
    int r = metrics(a, b, mode, m);
    if (r) return r;
    int k = 0;
    for (int p : M.coll.v) {
        HBPC& q = M.bpc[p];
        q.mm.push_back(m[k++]);
        if ((int)q.mm.size() > P.step_accum_merging) q.mm.erase(q.mm.begin());
        int notOnEdge = 0;
        for (int ref : q.list) if (stateH[ref] != AM_STATE_ONEDGE) notOnEdge++;
        int st;
        if (notOnEdge == 0) st = AM_STATE_ONEDGE;
        else if (notOnEdge >= 2) st = AM_STATE_CLEAR;
        else if (q.list.size() == 1) st = AM_STATE_CLEAR;
        else st = AM_STATE_ONEDGE;
        q.sh.push_back(st);
        if ((int)q.sh.size() > P.step_accum_merging) q.sh.erase(q.sh.begin());
    }
    return AM_OK;
}

// Sleeping.sleep's external-contact test per top-level body (Sleeping.java:65-73)
int Ctx::uploadExternalFlags() {
    std::vector<int> ext(host.cap, 0);
    for (int t : host.top)
        for (int p : M.bodyBpcs[t].v) {
            HBPC& q = M.bpc[p];
            if (!q.inCollection && !(pinned(host, q.a) || pinned(host, q.b))) { ext[t] = 1; break; }
        }
    cudaMemcpyAsync(extFlag, ext.data(), sizeof(int) * host.cap, cudaMemcpyHostToDevice, stream);
    return AM_OK;
}

// append store slots to the end of the current contact list (mode 3 copy)
int Ctx::appendFromStore(const std::vector<int>& slots, std::vector<int>& newIdx) {
    newIdx.clear();
    if (slots.empty()) return AM_OK;
    int live = nContacts + appended;
    int need = live + (int)slots.size();
    if (need > C[cur].cap) {   // grow, keeping the live contacts
        DContacts old = C[cur];
        int r = ensureContacts(need);
        if (r) return r;
        std::vector<int> idx(live);
        for (int k = 0; k < live; k++) idx[k] = k;
        if ((r = copyContacts(old, idx, C[cur], idx, 0))) return r;
    }
    for (size_t k = 0; k < slots.size(); k++) newIdx.push_back(live + (int)k);
    int r = copyContacts(I, slots, C[cur], newIdx, 3);
    if (r) return r;
    appended += (int)slots.size();
    for (int sl : slots) M.freeSlots.push_back(sl);
    return AM_OK;
}

int Ctx::ensurePairsKeep(int need) {
    if (need <= PR.cap) return AM_OK;
    DPairs old = PR;
    int r = ensurePairs(need);
    if (r) return r;
    cudaMemcpyAsync(PR.a, old.a, sizeof(int) * nPairs, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(PR.b, old.b, sizeof(int) * nPairs, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(PR.count, old.count, sizeof(int) * nPairs, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(PR.off, old.off, sizeof(int) * nPairs, cudaMemcpyDeviceToDevice, stream);
    return syncErr();
}

// pairs handed back by unmerge become groups of the full solve
int Ctx::flushAppendedPairs() {
    int k = (int)apA.size();
    if (k == 0) return AM_OK;
    int r = ensurePairsKeep(nPairs + k);
    if (r) return r;
    cudaMemcpyAsync(PR.a + nPairs, apA.data(), sizeof(int) * k, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(PR.b + nPairs, apB.data(), sizeof(int) * k, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(PR.count + nPairs, apCnt.data(), sizeof(int) * k, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(PR.off + nPairs, apOff.data(), sizeof(int) * k, cudaMemcpyHostToDevice, stream);
    r = syncErr();
    nPairs += k;
    apA.clear(); apB.clear(); apOff.clear(); apCnt.clear();
    return r;
}

// ---------------------------------------------------------------------------
// RigidBodySystem.advanceTime with merging (RigidBodySystem.java:102-185)
// RigidBodySystem.advanceTime with merging (RigidBodySystem.java:102-185), one
// phase at a time (the phases of am_step_phase, AM_MPHASE_*)
int Ctx::mergingPhase(int ph, double dt) {
    int r = AM_OK;
    double t;
    switch (ph) {
    case AM_MPHASE_COLLIDE:   // forces, updateContactsMap, collisionDetection, updateBodyPairContacts (:110-124)
        appended = 0;
        if ((r = beginStep(0))) return r;
        t = phaseNow();
        if ((r = collisionDetection())) return r;
        phaseAdd(AM_PHASE_DETECTION, t);
        return updateBodyPairContacts();
    case AM_MPHASE_WARM_START:   // warmStart, sleeping.wake (:126-132)
        t = phaseNow();
        if ((r = warmStart())) return r;
        phaseAdd(AM_PHASE_WARMSTART, t);
        if ((r = wake())) return r;
        cudaMemcpyAsync(host.flags.data(), B.flags, sizeof(int) * host.cap, cudaMemcpyDeviceToHost, stream);
        return syncErr();
    case AM_MPHASE_SINGLE_SWEEP:   // updateInCollections (:135)
        t = phaseNow();
        r = singleSweep(dt);
        phaseAdd(AM_PHASE_UPDATE_COLLECTIONS, t);
        return r;
    case AM_MPHASE_UNMERGE:   // accumulateForUnmerging, merging.unmerge, forces again (:138-147)
        t = phaseNow();
        if ((r = accumulateForUnmerging())) return r;
        if ((r = unmerge())) return r;
        if (appended) {   // contacts handed back by unmerge join the full solve (lambda = lambdaXwarm)
            nContacts += appended;
            appended = 0;
            if ((r = flushAppendedPairs())) return r;
        }
        if (mergingEvent && (r = beginStep(1))) return r;
        phaseAdd(AM_PHASE_UNMERGING, t);
        return AM_OK;
    case AM_MPHASE_SOLVE:   // redoWarmStart, solveLCP, clearBodyPairContacts (:150-157)
        if (nContacts > 0) {
            k_solve_bodies<<<(nContacts + 127) / 128, 128, 0, stream>>>(B, C[cur], nContacts);
            k_recompute_J<<<(nContacts + 127) / 128, 128, 0, stream>>>(B, C[cur], nContacts, 0);
            AM_LAUNCHED(2);
        }
        t = phaseNow();
        if ((r = solveLCP(dt, P.warm_start != 0))) return r;
        phaseAdd(AM_PHASE_LCP_SOLVE, t);
        return clearBodyPairContacts();
    case AM_MPHASE_ADVANCE:   // advanceBodiesVelocities, accumulateForMerging, advanceBodiesPositions (:160-166)
        advVel(dt);
        t = phaseNow();
        if ((r = accumulateForMerging())) return r;
        phaseAdd(AM_PHASE_MERGING, t);
        advPos(dt);
        return AM_OK;
    case AM_MPHASE_MERGE:   // merging.merge every stepsBetweenMergeEvents steps (:171-173)
        t = phaseNow();
        if ((totalSteps % P.steps_between_merge_events) == 0)
            if ((r = merge())) return r;
        phaseAdd(AM_PHASE_MERGING, t);
        return AM_OK;
    case AM_MPHASE_FINISH:   // sleeping.sleep (:176), counters
        if ((r = uploadExternalFlags())) return r;
        if ((r = sleepDecay())) return r;
        if ((r = readCounts())) return r;
        foldTiming();
        perf.steps++;
        return collectStats();
    }
    err = "unknown step phase";
    return AM_E_ARG;
}

int Ctx::stepWithMerging(double dt) {
    for (int ph = AM_MPHASE_COLLIDE; ph <= AM_MPHASE_FINISH; ph++) {
        int r = mergingPhase(ph, dt);
        if (r) return r;
    }
    return AM_OK;
}

// top-level list: a body is [id], a collection is [-1, members...]
int Ctx::getTopology(int* items, int* itemOff, int capItems, int* nTop, int* nItems) {
    int k = 0, t = 0;
    for (int b : host.top) {
        if (itemOff) itemOff[t] = k;
        if (host.flags[b] & F_COLLECTION) {
            if (items && k < capItems) items[k] = -1;
            k++;
            for (int s : host.subs[b]) { if (items && k < capItems) items[k] = s; k++; }
        } else {
            if (items && k < capItems) items[k] = b;
            k++;
        }
        t++;
    }
    if (itemOff) itemOff[t] = k;
    *nTop = t;
    *nItems = k;
    return k > capItems ? AM_E_CAPACITY : AM_OK;
}

}  // namespace am
