// state.cu -- snapshot and restore of a context's simulation state between
// steps (am_get_state / am_put_state).
//
// The reference keeps its state in Java objects (RigidBody fields, the
// contact pool, body-pair contacts with their histories, collections) and
// restores it by rebuilding them (RigidBodySystem.reset, RigidBodySystem.java:
// 390-426).  Here the state is split between the host (the body mirror with
// the collection structure, the insertion-ordered body-pair contacts and their
// motion-metric / contact-state histories) and the device (body arrays with the
// sleeping histories, the last step's contacts with their multipliers and
// warm-start copies, the store of contacts inside collections).  A snapshot
// is one byte blob holding all of it in a fixed order; restoring it into a
// context loaded with the same scene makes the next steps bit-identical to the
// steps that followed the snapshot.  Nothing recomputed at the start of every
// step (pairs, tree node centres, broad-phase prefilter, colouring) is kept.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "am_ctx.hpp"
#include "collections.hpp"

namespace am {

namespace {

const char MAGIC[4] = {'A', 'M', 'S', 'T'};
const int32_t VERSION = 1;

struct Header {
    char magic[4];
    int32_t version;
    int32_t n, cap, nNodes, nScenes;
    int32_t nContacts, nSlots, mergingEvent, kinSteps;
    int64_t totalSteps, mergeEvents, unmergeEvents;
};

struct Writer {
    std::vector<uint8_t> b;
    void raw(const void* p, size_t n) {
        const uint8_t* q = (const uint8_t*)p;
        b.insert(b.end(), q, q + n);
    }
    template <class T>
    void pod(const T& v) { raw(&v, sizeof(T)); }
    template <class T>
    void vec(const std::vector<T>& v) {
        int64_t n = (int64_t)v.size();
        pod(n);
        if (n) raw(v.data(), sizeof(T) * (size_t)n);
    }
    // n elements of device array d (waits for the copy: the next append may
    // move the buffer)
    template <class T>
    int dev(const T* d, size_t n, cudaStream_t s) {
        size_t off = b.size();
        b.resize(off + sizeof(T) * n);
        if (n && (cudaMemcpyAsync(b.data() + off, d, sizeof(T) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                  cudaStreamSynchronize(s) != cudaSuccess))
            return AM_E_CUDA;
        return AM_OK;
    }
};

struct Reader {
    const uint8_t* p;
    size_t n, off = 0;
    bool ok = true;
    bool raw(void* d, size_t k) {
        if (!ok || off + k > n) return ok = false;
        std::memcpy(d, p + off, k);
        off += k;
        return true;
    }
    template <class T>
    bool pod(T& v) { return raw(&v, sizeof(T)); }
    template <class T>
    bool vec(std::vector<T>& v, int64_t maxN = (int64_t)1 << 40) {
        int64_t k = 0;
        if (!pod(k) || k < 0 || k > maxN || off + sizeof(T) * (size_t)k > n) return ok = false;
        v.resize((size_t)k);
        return k == 0 || raw(v.data(), sizeof(T) * (size_t)k);
    }
    template <class T>
    bool dev(T* d, size_t k, cudaStream_t s) {
        if (!ok || off + sizeof(T) * k > n) return ok = false;
        if (k && cudaMemcpyAsync(d, p + off, sizeof(T) * k, cudaMemcpyHostToDevice, s) != cudaSuccess) return ok = false;
        off += sizeof(T) * k;
        return true;
    }
};

// every field of a contact buffer: (pointer, rows); each row holds `cap`
// entries, of which the first n are live
template <class F>
void contact_fields(DContacts& c, F f) {
    f(c.b1, 1); f(c.b2, 1); f(c.bv1, 1); f(c.bv2, 1); f(c.info, 1); f(c.pair, 1); f(c.state, 1); f(c.fresh, 1);
    f(c.sb1, 1); f(c.sb2, 1);
    f(c.f, 12); f(c.J, 36); f(c.cv, 1); f(c.pcv, 1); f(c.lam, 3); f(c.lamw, 3); f(c.bD, 6); f(c.Ia, 9);
    f(c.Ib, 9);
}

template <class F>
void body_fields(DBodies& B, F f) {
    f(B.type, 1); f(B.flags, 1); f(B.parent, 1); f(B.root, 1);
    f(B.x, 3); f(B.R, 9); f(B.v, 3); f(B.w, 3); f(B.mass, 1); f(B.minv, 1); f(B.jinv, 9); f(B.jinv0, 9);
    f(B.M, 9); f(B.M0, 9); f(B.force, 3); f(B.torque, 3); f(B.dv, 6); f(B.size, 3); f(B.radius, 1);
    f(B.friction, 1); f(B.restitution, 1); f(B.plane, 4); f(B.pp, 3); f(B.bbB, 24); f(B.hist, HIST);
    f(B.hist_n, 1); f(B.hist_h, 1); f(B.B2C, 12);
}

}  // namespace

int Ctx::getState(std::vector<uint8_t>& out) {
    if (!stream || host.cap == 0) { err = "no scene loaded"; return AM_E_STATE; }
    Writer w;
    Header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, MAGIC, 4);
    h.version = VERSION;
    h.n = host.n;
    h.cap = host.cap;
    h.nNodes = N.n;
    h.nScenes = nScenes;
    h.nContacts = nContacts;
    h.nSlots = M.nSlots;
    h.mergingEvent = mergingEvent ? 1 : 0;
    h.kinSteps = kinSteps;
    h.totalSteps = totalSteps;
    h.mergeEvents = mergeEvents;
    h.unmergeEvents = unmergeEvents;
    w.pod(h);
    // host mirror of the bodies and the collection structure
    const HostWorld& hw = host;
    w.vec(hw.type); w.vec(hw.flags); w.vec(hw.parent); w.vec(hw.root);
    w.vec(hw.x); w.vec(hw.R); w.vec(hw.v); w.vec(hw.w); w.vec(hw.mass); w.vec(hw.minv); w.vec(hw.jinv);
    w.vec(hw.jinv0); w.vec(hw.M); w.vec(hw.M0); w.vec(hw.size); w.vec(hw.radius); w.vec(hw.friction);
    w.vec(hw.restitution); w.vec(hw.plane); w.vec(hw.pp); w.vec(hw.bbB); w.vec(hw.B2C); w.vec(hw.top);
    w.vec(hw.nbb);
    w.pod((int64_t)hw.subs.size());
    for (const auto& s : hw.subs) w.vec(s);
    // body-pair contacts (CollisionProcessor.bodyPairContacts and the per-body sets)
    w.pod((int64_t)M.bpc.size());
    for (const HBPC& p : M.bpc) {
        w.pod(p.a);
        w.pod(p.b);
        w.vec(p.list);
        w.vec(p.mm);
        w.vec(p.sh);
        w.pod((int32_t)p.inCollection);
        w.pod((int32_t)p.checked);
    }
    w.vec(M.coll.v);
    w.pod((int64_t)M.bodyBpcs.size());
    for (const OSetI& s : M.bodyBpcs) w.vec(s.v);
    std::vector<uint64_t> keys;
    std::vector<int32_t> vals;
    for (const auto& kv : M.index) { keys.push_back(kv.first); vals.push_back(kv.second); }
    w.vec(keys);
    w.vec(vals);
    w.vec(M.freeSlots);
    // device: bodies, sleep / external flags, the last step's contacts, the collection store
    int r = AM_OK;
    const size_t cap = (size_t)host.cap;
    body_fields(B, [&](auto* d, int rows) { if (!r) r = w.dev(d, rows * cap, stream); });
    if (!r) r = w.dev(wakeFlag, cap, stream);
    if (!r) r = w.dev(extFlag, cap, stream);
    DContacts& c = C[cur];
    const size_t nc = (size_t)nContacts;
    contact_fields(c, [&](auto* d, int rows) {
        for (int q = 0; q < rows && !r; q++) r = w.dev(d + (size_t)q * c.cap, nc, stream);
    });
    const size_t ns = (size_t)M.nSlots;
    if (ns)
        contact_fields(I, [&](auto* d, int rows) {
            for (int q = 0; q < rows && !r; q++) r = w.dev(d + (size_t)q * I.cap, ns, stream);
        });
    if (r) { err = "state download"; return r; }
    if ((r = syncErr())) return r;
    out.swap(w.b);
    return AM_OK;
}

int Ctx::putState(const uint8_t* in, size_t size) {
    if (!stream || host.cap == 0) { err = "no scene loaded"; return AM_E_STATE; }
    Reader rd{in, size};
    Header h;
    if (!rd.pod(h) || std::memcmp(h.magic, MAGIC, 4) != 0 || h.version != VERSION) {
        err = "not a state snapshot of this library version";
        return AM_E_ARG;
    }
    if (h.n != host.n || h.cap != host.cap || h.nNodes != N.n || h.nScenes != nScenes) {
        err = "the snapshot was taken from another scene (body, slot, node or scene counts differ)";
        return AM_E_STATE;
    }
    if (h.nContacts < 0 || h.nSlots < 0) { err = "malformed snapshot"; return AM_E_ARG; }
    HostWorld hw = host;
    const int64_t lim = (int64_t)host.cap * 64 + 4096;
    bool ok = rd.vec(hw.type, lim) && rd.vec(hw.flags, lim) && rd.vec(hw.parent, lim) && rd.vec(hw.root, lim) &&
              rd.vec(hw.x, lim) && rd.vec(hw.R, lim) && rd.vec(hw.v, lim) && rd.vec(hw.w, lim) &&
              rd.vec(hw.mass, lim) && rd.vec(hw.minv, lim) && rd.vec(hw.jinv, lim) && rd.vec(hw.jinv0, lim) &&
              rd.vec(hw.M, lim) && rd.vec(hw.M0, lim) && rd.vec(hw.size, lim) && rd.vec(hw.radius, lim) &&
              rd.vec(hw.friction, lim) && rd.vec(hw.restitution, lim) && rd.vec(hw.plane, lim) &&
              rd.vec(hw.pp, lim) && rd.vec(hw.bbB, lim) && rd.vec(hw.B2C, lim) && rd.vec(hw.top, lim) &&
              rd.vec(hw.nbb, lim);
    int64_t nsub = 0;
    ok = ok && rd.pod(nsub) && nsub == (int64_t)host.cap;
    if (ok) {
        hw.subs.assign((size_t)nsub, {});
        for (auto& s : hw.subs) ok = ok && rd.vec(s, lim);
    }
    // the body arrays keep their sizes (cap slots)
    ok = ok && hw.type.size() == host.type.size() && hw.x.size() == host.x.size() && hw.R.size() == host.R.size() &&
         hw.top.size() <= (size_t)host.cap;
    HostMerge hm;
    int64_t nb = 0;
    ok = ok && rd.pod(nb) && nb >= 0 && nb <= lim * 8;
    if (ok) {
        hm.bpc.resize((size_t)nb);
        for (HBPC& p : hm.bpc) {
            int32_t ic = 0, ck = 0;
            ok = ok && rd.pod(p.a) && rd.pod(p.b) && rd.vec(p.list, lim) && rd.vec(p.mm, lim) && rd.vec(p.sh, lim) &&
                 rd.pod(ic) && rd.pod(ck);
            p.inCollection = ic != 0;
            p.checked = ck != 0;
        }
    }
    std::vector<int> collv;
    ok = ok && rd.vec(collv, lim * 8);
    int64_t nbs = 0;
    ok = ok && rd.pod(nbs) && nbs == (int64_t)host.cap;
    if (ok) {
        hm.bodyBpcs.assign((size_t)nbs, OSetI());
        for (OSetI& s : hm.bodyBpcs) {
            std::vector<int> v;
            ok = ok && rd.vec(v, lim * 8);
            for (int x : v) s.add(x);
        }
    }
    for (int x : collv) hm.coll.add(x);
    std::vector<uint64_t> keys;
    std::vector<int32_t> vals;
    ok = ok && rd.vec(keys, lim * 8) && rd.vec(vals, lim * 8) && keys.size() == vals.size();
    if (ok)
        for (size_t k = 0; k < keys.size(); k++) hm.index[keys[k]] = vals[k];
    ok = ok && rd.vec(hm.freeSlots, lim * 8);
    hm.nSlots = h.nSlots;
    if (!ok) { err = "malformed snapshot"; return AM_E_ARG; }
    // the device part must be exactly what the header promises, checked
    // before any device array is written
    {
        size_t need = 0;
        body_fields(B, [&](auto* d, int rows) { need += sizeof(*d) * rows * (size_t)host.cap; });
        need += 2 * sizeof(int) * (size_t)host.cap;
        size_t per = 0;
        contact_fields(C[cur], [&](auto* d, int rows) { per += sizeof(*d) * rows; });
        need += per * ((size_t)h.nContacts + (size_t)h.nSlots);
        if (rd.off + need != size) { err = "malformed snapshot (size)"; return AM_E_ARG; }
    }
    // device arrays
    int r = AM_OK;
    if ((r = ensureContacts(std::max(h.nContacts, 1)))) return r;
    if (h.nSlots && (r = ensureStore(h.nSlots))) return r;
    const size_t cap = (size_t)host.cap;
    body_fields(B, [&](auto* d, int rows) { ok = ok && rd.dev(d, rows * cap, stream); });
    ok = ok && rd.dev(wakeFlag, cap, stream) && rd.dev(extFlag, cap, stream);
    DContacts& c = C[cur];
    const size_t nc = (size_t)h.nContacts;
    contact_fields(c, [&](auto* d, int rows) {
        for (int q = 0; q < rows; q++) ok = ok && rd.dev(d + (size_t)q * c.cap, nc, stream);
    });
    const size_t ns = (size_t)h.nSlots;
    if (ns)
        contact_fields(I, [&](auto* d, int rows) {
            for (int q = 0; q < rows; q++) ok = ok && rd.dev(d + (size_t)q * I.cap, ns, stream);
        });
    if ((r = syncErr())) return r;   // the host buffer is read by the copies until here
    if (!ok || rd.off != size) { err = "malformed snapshot (device part)"; return AM_E_ARG; }
    host = hw;
    host.P = &P;
    M = hm;
    nContacts = h.nContacts;
    nPairs = 0;
    totalSteps = (int)h.totalSteps;
    mergingEvent = h.mergingEvent != 0;
    kinSteps = h.kinSteps;
    mergeEvents = h.mergeEvents;
    unmergeEvents = h.unmergeEvents;
    // the device's top-level list and collection members follow the host
    // mirror (flags and parent stay as the snapshot's device copies: the
    // device holds the sleeping bits)
    std::vector<int> nbbv(host.nbb.begin(), host.nbb.end());
    cudaMemcpyAsync(nbbDev, nbbv.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream);
    ntop = (int)host.top.size();
    if (ntop) cudaMemcpyAsync(top, host.top.data(), sizeof(int) * ntop, cudaMemcpyHostToDevice, stream);
    std::vector<int> so(cap + 1, 0), si;
    for (size_t b = 0; b < cap; b++) {
        so[b] = (int)si.size();
        if (host.flags[b] & F_COLLECTION)
            for (int q : host.subs[b]) si.push_back(q);
    }
    so[cap] = (int)si.size();
    if (si.size() > cap) { err = "malformed snapshot (collection members)"; return AM_E_ARG; }
    nSubIds = (int)si.size();
    cudaMemcpyAsync(subOff, so.data(), sizeof(int) * (cap + 1), cudaMemcpyHostToDevice, stream);
    if (!si.empty()) cudaMemcpyAsync(subIds, si.data(), sizeof(int) * si.size(), cudaMemcpyHostToDevice, stream);
    return syncErr();
}

}  // namespace am
