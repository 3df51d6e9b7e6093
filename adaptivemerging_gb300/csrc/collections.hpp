// collections.hpp -- host-side world mirror and the step context.
//
// HostWorld keeps the per-body records that the host needs to own: the
// top-level body list (RigidBodySystem.bodies), collection membership and the
// derived mass properties computed at load time (XMLParser.java:360-447,
// RigidBody.java:182-206, PlaneRigidBody.java:49-57).  Contacts, pairs and
// the per-step state live on the device.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"

namespace am {

inline double __longlong_as_double_host(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

struct HostWorld {
    int n = 0;       // scene bodies
    int cap = 0;     // body slots (scene + collections)
    const am_params* P = nullptr;
    std::vector<int> type, flags, parent, root;
    std::vector<double> x, R, v, w, mass, minv, jinv, jinv0, M, M0, size, radius, friction, restitution,
        plane, pp, bbB, B2C;
    std::vector<int> top;                 // top-level list in reference order
    std::vector<std::vector<int>> subs;   // collection members in order

    bool anyMerging() const { return P && P->enable_merging; }

    void init(const am_scene& s, const am_params& p) {
        using namespace amd;
        P = &p;
        n = s.n_bodies;
        cap = n + n / 2 + 16;
        type.assign(cap, -1); flags.assign(cap, 0); parent.assign(cap, -1); root.assign(cap, -1);
        x.assign(3 * cap, 0); R.assign(9 * cap, 0); v.assign(3 * cap, 0); w.assign(3 * cap, 0);
        mass.assign(cap, 0); minv.assign(cap, 0); jinv.assign(9 * cap, 0); jinv0.assign(9 * cap, 0);
        M.assign(9 * cap, 0); M0.assign(9 * cap, 0); size.assign(3 * cap, 0); radius.assign(cap, 0);
        friction.assign(cap, 0.8); restitution.assign(cap, 0); plane.assign(4 * cap, 0); pp.assign(3 * cap, 0);
        bbB.assign(24 * cap, 0); B2C.assign(12 * cap, 0);
        subs.assign(cap, {});
        top.clear();
        for (int i = 0; i < n; i++) {
            type[i] = s.type[i];
            friction[i] = s.friction[i];
            restitution[i] = s.restitution[i];
            root[i] = s.body_root[i];
            m3 Id = ident();
            stm(&R[9 * i], Id);
            top.push_back(i);
            if (type[i] == AM_PLANE) {   // PlaneRigidBody: pinned, massless, x at the origin
                v3 nn = mk(s.shape[4 * i], s.shape[4 * i + 1], s.shape[4 * i + 2]);
                normalize(nn);
                v3 q = mk(s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]);
                plane[4 * i] = nn.x; plane[4 * i + 1] = nn.y; plane[4 * i + 2] = nn.z;
                plane[4 * i + 3] = -(q.x * nn.x + q.y * nn.y + q.z * nn.z);
                stv(&pp[3 * i], q);
                flags[i] = F_PINNED;
                continue;
            }
            for (int k = 0; k < 3; k++) {
                x[3 * i + k] = s.x[3 * i + k];
                v[3 * i + k] = s.v[3 * i + k];
                w[3 * i + k] = s.omega[3 * i + k];
            }
            for (int k = 0; k < 9; k++) { R[9 * i + k] = s.R[9 * i + k]; M0[9 * i + k] = s.inertia[9 * i + k]; }
            mass[i] = s.mass[i];
            bool pinned = s.pinned[i] != 0;
            flags[i] = pinned ? F_PINNED : 0;
            v3 ll, ur;
            if (type[i] == AM_BOX) {
                v3 sz = mk(s.shape[4 * i], s.shape[4 * i + 1], s.shape[4 * i + 2]);
                stv(&size[3 * i], sz);
                v3 h = scale(0.5, sz);
                radius[i] = length(h);
                ll = mk(-h.x, -h.y, -h.z); ur = h;
            } else if (type[i] == AM_SPHERE) {
                double r = s.shape[4 * i];
                ll = mk(-r, -r, -r); ur = mk(r, r, r);
            } else {   // sphere tree: box of the leaf spheres
                ll = mk(1e300, 1e300, 1e300); ur = mk(-1e300, -1e300, -1e300);
                std::vector<int> st{s.body_root[i]};
                while (!st.empty()) {
                    int k = st.back(); st.pop_back();
                    if (s.node_child0[k] >= 0) {
                        for (int q = 0; q < s.node_nchild[k]; q++) st.push_back(s.node_child0[k] + q);
                        continue;
                    }
                    v3 c = mk(s.node_c[3 * k], s.node_c[3 * k + 1], s.node_c[3 * k + 2]);
                    double r = s.node_r[k];
                    ll.x = std::min(c.x - r, ll.x); ll.y = std::min(c.y - r, ll.y); ll.z = std::min(c.z - r, ll.z);
                    ur.x = std::max(c.x + r, ur.x); ur.y = std::max(c.y + r, ur.y); ur.z = std::max(c.z + r, ur.z);
                }
            }
            v3 corners[8] = {mk(ll.x, ll.y, ll.z), mk(ll.x, ll.y, ur.z), mk(ll.x, ur.y, ll.z), mk(ll.x, ur.y, ur.z),
                             mk(ur.x, ll.y, ll.z), mk(ur.x, ll.y, ur.z), mk(ur.x, ur.y, ll.z), mk(ur.x, ur.y, ur.z)};
            for (int k = 0; k < 8; k++) stv(&bbB[24 * i + 3 * k], corners[k]);
            m3 Ri = ldm(&R[9 * i]), M0i = ldm(&M0[9 * i]);
            stm(&M[9 * i], rm0rt(Ri, M0i));
            if (!pinned) {
                minv[i] = 1.0 / mass[i];
                m3 J0;
                if (!invert3(M0i, J0)) J0 = zero3();
                stm(&jinv0[9 * i], J0);
                stm(&jinv[9 * i], rm0rt(Ri, J0));
            }
        }
    }
};

// The step context behind the C ABI.
struct Ctx {
    am_params P;
    std::string err;
    HostWorld host;
    cudaStream_t stream = nullptr;
    DBodies B;
    DNodes N;
    DContacts C[2];
    int cur = 0;
    DPairs PR;
    DHash H;
    Scratch SC;
    DCount* dc = nullptr;
    DCount* hc = nullptr;
    int* top = nullptr;
    int* subOff = nullptr;
    int* subIds = nullptr;
    int* rowCount = nullptr;
    int* rowOff = nullptr;
    int* candA = nullptr;
    int* candB = nullptr;
    int candCap = 0;
    int* wakeFlag = nullptr;
    int* extFlag = nullptr;
    int* bodyMax = nullptr;   // 64-bit slots reinterpreted (allocated as 2 ints per body below)
    int* colourOf = nullptr;
    int* groupOrder = nullptr;
    int* colourCnt = nullptr;
    int* colourOff = nullptr;
    int* colourFill = nullptr;
    static const int MAXC = 256;
    int coopBlocks = 0;
    int nScene = 0, ntop = 0, nContacts = 0, nPrev = 0, nPairs = 0;
    int totalSteps = 0;
    bool mergingEvent = false;
    am_solve_stats stats{};
    std::vector<void*> allocs;

    explicit Ctx(const am_params& p);
    ~Ctx();
    void release();
    template <class T>
    int alloc(T** p, size_t n);
    int allocContacts(DContacts& c, int cap);
    int ensureContacts(int need);
    int ensurePairs(int need);
    int ensureScratch(int need);
    int ensureCand(int need);
    int setScene(const am_scene& s);
    int uploadBodies(bool full);
    int uploadTopology();
    int syncErr();
    int readCounts();
    void gravityDir(double g[3]) const;
    int beginStep(int mode);
    int collisionDetection();
    int warmStart();
    int wake();
    int runPGS(int nc, const int* order, int iters, bool inColl, double dt, bool redoWarm);
    int solveLCP(double dt, bool redoWarm);
    int finishStep(double dt);
    int step(double dt);
    int stepWithMerging(double dt);
    int collectStats();
    int getBodies(am_body_state* out);
    int getContacts(am_contacts* out, int capacity, int* n);
};

const void* pgs_coloured_kernel();

}  // namespace am
