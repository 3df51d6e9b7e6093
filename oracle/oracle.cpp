// oracle.cpp -- TEST INFRASTRUCTURE ONLY (see oracle.hpp).  Restates the
// reference's 3D step; every function cites the Java it follows (paths are
// relative to src/mergingBodies3D in the reference project).
#include "oracle.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "sincos.hpp"

namespace orc {

// java.lang.Math.max / Math.min, including the signed-zero and NaN rules.
static inline double jmax(double a, double b) {
    if (a != a) return a;
    if (a == 0.0 && b == 0.0 && std::signbit(a)) return b;
    return (a >= b) ? a : b;
}
static inline double jmin(double a, double b) {
    if (a != a) return a;
    if (a == 0.0 && b == 0.0 && std::signbit(b)) return b;
    return (a <= b) ? a : b;
}

// ---------------------------------------------------------------------------
// Scene loading: XMLParser.java:360-447 (box, plane, sphere), 449-539 (mesh /
// sphere tree), RigidBody.java:182-206 (constructor), PlaneRigidBody.java:49-57.
void World::init(const am_params& p, const am_scene& s) {
    P = p;
    nScene = s.n_bodies;
    nodes.resize(s.n_nodes);
    for (int k = 0; k < s.n_nodes; k++) {
        Node& n = nodes[k];
        n.cB = V3(s.node_c[3 * k], s.node_c[3 * k + 1], s.node_c[3 * k + 2]);
        n.r = s.node_r[k];
        n.child0 = s.node_child0[k];
        n.nchild = s.node_nchild[k];
        n.id = k;
    }
    for (int i = 0; i < s.n_bodies; i++) {
        store.emplace_back();
        Body& b = store.back();
        b.id = i;
        b.type = s.type[i];
        b.friction = s.friction[i];
        b.restitution = s.restitution[i];
        b.theta = M3::identity();
        if (b.type == AM_PLANE) {
            // PlaneRigidBody(p, n): pinned, zero mass, x stays at the origin
            V3 n(s.shape[4 * i], s.shape[4 * i + 1], s.shape[4 * i + 2]);
            vnormalize(n);
            b.pn = n;
            b.pp = V3(s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]);
            b.pd = -(b.pp.x * n.x + b.pp.y * n.y + b.pp.z * n.z);
            b.pinned = true;
            bodies.push_back(&b);
            continue;
        }
        b.x = V3(s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]);
        M3 R;
        double* pr = &R.m00;
        for (int k = 0; k < 9; k++) pr[k] = s.R[9 * i + k];
        b.theta = R;
        b.v = V3(s.v[3 * i], s.v[3 * i + 1], s.v[3 * i + 2]);
        b.omega = V3(s.omega[3 * i], s.omega[3 * i + 1], s.omega[3 * i + 2]);
        b.massLinear = s.mass[i];
        M3 I;
        double* pi = &I.m00;
        for (int k = 0; k < 9; k++) pi[k] = s.inertia[9 * i + k];
        b.massAngular0 = I;
        b.pinned = s.pinned[i] != 0;
        if (b.type == AM_BOX) {
            V3 sz(s.shape[4 * i], s.shape[4 * i + 1], s.shape[4 * i + 2]);
            b.size = sz;
            V3 h = vscale(0.5, sz);
            b.bbB = {V3(-h.x, -h.y, -h.z), V3(-h.x, -h.y, h.z), V3(-h.x, h.y, -h.z), V3(-h.x, h.y, h.z),
                     V3(h.x, -h.y, -h.z), V3(h.x, -h.y, h.z), V3(h.x, h.y, -h.z), V3(h.x, h.y, h.z)};
            b.radius = vlength(h);
        } else if (b.type == AM_SPHERE) {
            double r = s.shape[4 * i];
            b.bbB = {V3(-r, -r, -r), V3(-r, -r, r), V3(-r, r, -r), V3(-r, r, r),
                     V3(r, -r, -r), V3(r, -r, r), V3(r, r, -r), V3(r, r, r)};
        } else if (b.type == ORC_COMPOSITE) {
            // createComposite's box of the sub-bodies' corners, in its own corner
            // order (XMLParser.java:280-306)
            const double* q = s.bbox ? s.bbox + 6 * i : nullptr;
            if (q)
                b.bbB = {V3(q[0], q[1], q[2]), V3(q[0], q[1], q[5]), V3(q[0], q[4], q[2]), V3(q[0], q[4], q[5]),
                         V3(q[3], q[4], q[5]), V3(q[3], q[1], q[2]), V3(q[3], q[1], q[5]), V3(q[3], q[4], q[2])};
        } else if (s.bbox && std::isfinite(s.bbox[6 * i]) && std::isfinite(s.bbox[6 * i + 1]) &&
                   std::isfinite(s.bbox[6 * i + 2]) && std::isfinite(s.bbox[6 * i + 3]) &&
                   std::isfinite(s.bbox[6 * i + 4]) && std::isfinite(s.bbox[6 * i + 5])) {
            // a mesh body: the box of its mesh's vertices (XMLParser.java:474-493)
            const double* q = s.bbox + 6 * i;
            b.bbB = {V3(q[0], q[1], q[2]), V3(q[0], q[1], q[5]), V3(q[0], q[4], q[2]), V3(q[0], q[4], q[5]),
                     V3(q[3], q[1], q[2]), V3(q[3], q[1], q[5]), V3(q[3], q[4], q[2]), V3(q[3], q[4], q[5])};
        } else {  // sphere tree without a mesh (a clump): the box of its leaf spheres
            V3 ll(1e300, 1e300, 1e300), ur(-1e300, -1e300, -1e300);
            std::vector<int> st{s.body_root[i]};
            while (!st.empty()) {
                int k = st.back(); st.pop_back();
                if (s.node_child0[k] >= 0) {
                    for (int q = 0; q < s.node_nchild[k]; q++) st.push_back(s.node_child0[k] + q);
                    continue;
                }
                V3 c(s.node_c[3 * k], s.node_c[3 * k + 1], s.node_c[3 * k + 2]);
                double r = s.node_r[k];
                ll.x = std::min(c.x - r, ll.x); ll.y = std::min(c.y - r, ll.y); ll.z = std::min(c.z - r, ll.z);
                ur.x = std::max(c.x + r, ur.x); ur.y = std::max(c.y + r, ur.y); ur.z = std::max(c.z + r, ur.z);
            }
            b.bbB = {V3(ll.x, ll.y, ll.z), V3(ll.x, ll.y, ur.z), V3(ll.x, ur.y, ll.z), V3(ll.x, ur.y, ur.z),
                     V3(ur.x, ll.y, ll.z), V3(ur.x, ll.y, ur.z), V3(ur.x, ur.y, ll.z), V3(ur.x, ur.y, ur.z)};
        }
        b.root = s.body_root[i];
        if (!b.pinned) {
            b.minv = 1.0 / b.massLinear;
            minvert(b.massAngular0, b.jinv0);
            b.massAngular = rm0rt(b.theta, b.massAngular0);
            b.jinv = rm0rt(b.theta, b.jinv0);
        } else {
            b.minv = 0;
            b.massAngular = rm0rt(b.theta, b.massAngular0);
        }
        bodies.push_back(&b);
    }
    for (int k = 0; k < s.n_subs; k++)
        if (addCompositeSub(s.sub_parent[k], s.sub_type[k], s.sub_shape + 4 * k, s.sub_R + 9 * k, s.sub_t + 3 * k))
            badSubs++;
    for (int i = 0; i < s.n_bodies; i++) {
        int r0 = s.body_root[i];
        if (r0 < 0) continue;
        std::vector<int> st{r0};
        while (!st.empty()) {
            int q = st.back(); st.pop_back();
            nodes[q].body = &store[i];
            for (int c = 0; c < nodes[q].nchild; c++) st.push_back(nodes[q].child0 + c);
        }
    }
}

// A sub-body of composite `parent` (XMLParser.createComposite, :180-352): a box
// (shape = size) or a sphere (shape[0] = r, one BV leaf at its centre, as
// createSphere builds it), with transformB2C = (R, t), its pose in the
// composite's frame.  Sub-bodies never enter the body list: collisions with
// the composite run on them, placed from the parent first.
int World::addCompositeSub(int parent, int type, const double* shape, const double* R, const double* t) {
    if (parent < 0 || parent >= nScene || store[parent].type != ORC_COMPOSITE) return -1;
    if (type != AM_BOX && type != AM_SPHERE) return -1;
    Body* p = &store[parent];
    subStore.emplace_back();
    Body* b = &subStore.back();
    b->id = ORC_SUB_ID0 + (int)subStore.size() - 1;
    b->type = type;
    b->friction = p->friction;
    b->restitution = p->restitution;
    M3 Rm;
    double* pr = &Rm.m00;
    for (int k = 0; k < 9; k++) pr[k] = R[k];
    b->B2Cc = RT{Rm, V3(t[0], t[1], t[2])};
    b->compParent = p;
    if (type == AM_BOX) {
        b->size = V3(shape[0], shape[1], shape[2]);
        b->radius = vlength(vscale(0.5, b->size));
    } else {
        Node n;
        n.cB = V3();
        n.r = shape[0];
        n.body = b;
        n.id = (int)nodes.size();
        nodes.push_back(n);
        b->root = n.id;
        // nodes[k].body of the scene's trees point into `store`, which does not move
    }
    p->subs.push_back(b);
    RT T = rt_mult(p->T(), b->B2Cc);
    b->theta = T.R;
    b->x = T.t;
    return 0;
}

// RigidBodyGeomComposite.updateBodyPositionsFromParent (:32-36): transformB2W =
// parent.transformB2W * transformB2C.  The reference runs it in narrowPhase
// before each composite's sub-body collisions; a parent does not move during
// detection, so once before the pass gives the same poses.
void World::updateCompositeSubs() {
    for (Body& b : subStore) {
        RT T = rt_mult(b.compParent->T(), b.B2Cc);
        b.theta = T.R;
        b.x = T.t;
    }
}

Contact* World::newContact() {  // ContactPool.get (ContactPool.java:46-53)
    pool[cur].emplace_back();
    return &pool[cur].back();
}

// ---------------------------------------------------------------------------
// Contact.set + computeJacobian (Contact.java:159-255)
static void computeJacobian(Contact* c, bool inColl, const V3& pW, const V3& n, const V3& t1, const V3& t2) {
    Body* b1 = (c->body1->parent && !inColl) ? c->body1->parent : c->body1;
    Body* b2 = (c->body2->parent && !inColl) ? c->body2->parent : c->body2;
    V3 r1 = vsub(pW, b1->x);
    V3 r2 = vsub(pW, b2->x);
    c->jna_v = vscale(-1, n);
    c->jna_w = vcross(n, r1);
    c->jnb_v = n;
    c->jnb_w = vcross(r2, n);
    c->jt1a_v = vscale(-1, t1);
    c->jt1a_w = vcross(t1, r1);
    c->jt1b_v = t1;
    c->jt1b_w = vcross(r2, t1);
    c->jt2a_v = vscale(-1, t2);
    c->jt2a_w = vcross(t2, r1);
    c->jt2b_v = t2;
    c->jt2b_w = vcross(r2, t2);
}

// Contact.computeJacobian(boolean) (Contact.java:265-271): frame from body 1
static void recomputeJacobian(Contact* c, bool inColl) {
    RT T = c->body1->T();
    V3 p = rt_point(T, c->cB1);
    V3 n = rt_vec(T, c->nB1);
    V3 t1 = rt_vec(T, c->t1B1);
    V3 t2 = rt_vec(T, c->t2B1);
    computeJacobian(c, inColl, p, n, t1, t2);
}

void World::emit(Body* b1, Body* b2, const V3& pW, const V3& nW, int bv1, int bv2, int info, double cv) {
    Contact* c = newContact();
    c->state = CLEAR;
    // a composite's sub-body hands the contact to its composite and stays as
    // the contact's csb for the warm-start key (Contact.java:167-181)
    c->csb1 = c->csb2 = -1;
    if (b1->compParent) { c->csb1 = b1->id; b1 = b1->compParent; }
    if (b2->compParent) { c->csb2 = b2->id; b2 = b2->compParent; }
    c->body1 = b1;
    c->body2 = b2;
    c->info = info;
    c->bv1 = bv1;
    c->bv2 = bv2;
    c->cv = cv;
    c->prevCv = 0;
    c->l0 = c->l1 = c->l2 = 0;
    c->l0w = c->l1w = c->l2w = 0;
    double anx = std::fabs(nW.x), any = std::fabs(nW.y), anz = std::fabs(nW.z);
    V3 t1;
    if (anx < any && anx < anz) t1 = V3(1, 0, 0);
    else if (any < anz) t1 = V3(0, 1, 0);
    else t1 = V3(0, 0, 1);
    V3 t2 = vcross(nW, t1);
    vnormalize(t2);
    t1 = vcross(t2, nW);
    computeJacobian(c, false, pW, nW, t1, t2);
    RT T = b1->T();
    c->cB1 = rt_inv_point(T, pW);
    c->nB1 = mtxv(T.R, nW);
    c->t1B1 = mtxv(T.R, t1);
    c->t2B1 = mtxv(T.R, t2);
    c->bn = c->bt1 = c->bt2 = 0;
    c->D00 = c->D11 = c->D22 = 0;
    c->fresh = true;
    contacts.push_back(c);
}

// ---------------------------------------------------------------------------
// BoxPlane.dBoxPlane (collision/BoxPlane.java:27-52)
void World::boxPlane(Body* box, Body* plane) {
    const V3& n = plane->pn;
    double d = plane->pd;
    if (box->x.x * n.x + box->x.y * n.y + box->x.z * n.z + d > box->radius) return;
    V3 p = vscale(0.5, box->size);
    RT T = box->T();
    static const int sg[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                 {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    for (int k = 0; k < 8; k++) {
        V3 q(sg[k][0] > 0 ? p.x : -p.x, sg[k][1] > 0 ? p.y : -p.y, sg[k][2] > 0 ? p.z : -p.z);
        q = rt_point(T, q);
        double s = q.x * n.x + q.y * n.y + q.z * n.z + d;
        if (s < 0) emit(plane, box, q, n, AM_BV_NULL, AM_BV_NULL, k, s);  // plane is body 1
    }
}

// BoxSphere.dBoxSphereTest (collision/BoxSphere.java:156-233)
bool World::boxSphereTest(Body* box, const V3& c, double r) {
    if (pdist(c, box->x) > box->radius + r) return false;
    V3 p = vscale(0.5, box->size);
    V3 cB = rt_inv_point(box->T(), c);
    if (cB.x - p.x > r) return false;
    if (-p.x - cB.x > r) return false;
    if (cB.y - p.y > r) return false;
    if (-p.y - cB.y > r) return false;
    if (cB.z - p.z > r) return false;
    if (-p.z - cB.z > r) return false;
    static const int sg[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                 {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    for (int k = 0; k < 8; k++) {
        V3 q(sg[k][0] > 0 ? p.x : -p.x, sg[k][1] > 0 ? p.y : -p.y, sg[k][2] > 0 ? p.z : -p.z);
        if (pdist(cB, q) - r < 0) return true;
    }
    if (-p.x <= cB.x && cB.x <= p.x) {
        if (cB.y >= p.y && cB.z >= p.z) { if (vlength(V3(0, cB.y - p.y, cB.z - p.z)) - r < 0) return true; }
        else if (cB.y <= -p.y && cB.z >= p.z) { if (vlength(V3(0, cB.y + p.y, cB.z - p.z)) - r < 0) return true; }
        else if (cB.y >= p.y && cB.z <= -p.z) { if (vlength(V3(0, cB.y - p.y, cB.z + p.z)) - r < 0) return true; }
        else if (cB.y <= -p.y && cB.z <= -p.z) { if (vlength(V3(0, cB.y + p.y, cB.z + p.z)) - r < 0) return true; }
    }
    if (-p.y <= cB.y && cB.y <= p.y) {
        if (cB.x >= p.x && cB.z >= p.z) { if (vlength(V3(cB.x - p.x, 0, cB.z - p.z)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.z >= p.z) { if (vlength(V3(cB.x + p.x, 0, cB.z - p.z)) - r < 0) return true; }
        else if (cB.x >= p.x && cB.z <= -p.z) { if (vlength(V3(cB.x - p.x, 0, cB.z + p.z)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.z <= -p.z) { if (vlength(V3(cB.x + p.x, 0, cB.z + p.z)) - r < 0) return true; }
    }
    if (-p.z < cB.z && cB.z < p.z) {
        if (cB.x >= p.x && cB.y >= p.y) { if (vlength(V3(cB.x - p.x, cB.y - p.y, 0)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.y >= p.y) { if (vlength(V3(cB.x + p.x, cB.y - p.y, 0)) - r < 0) return true; }
        else if (cB.x >= p.x && cB.y <= -p.y) { if (vlength(V3(cB.x - p.x, cB.y + p.y, 0)) - r < 0) return true; }
        else if (cB.x <= -p.x && cB.y <= -p.y) { if (vlength(V3(cB.x + p.x, cB.y + p.y, 0)) - r < 0) return true; }
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

// BoxSphere.dBoxSphere with test1/test2 (collision/BoxSphere.java:58-144, 242-275)
void World::boxSphere(Body* box, Body* sph, const V3& c, double r) {
    V3 p = vscale(0.5, box->size);
    V3 cB = rt_inv_point(box->T(), c);
    double depth = 1;
    V3 pos, nrm;
    auto test1 = [&](const V3& q) {
        double s = pdist(cB, q) - r;
        if (s > 0) return;
        if (s < depth) { pos = q; nrm = vsub(cB, q); vnormalize(nrm); depth = s; }
    };
    auto test2 = [&](double s, double px, double py, double pz, double nx, double ny, double nz) {
        if (s > 0) return;
        if (s < depth) { pos = V3(px, py, pz); nrm = V3(nx, ny, nz); depth = s; }
    };
    static const int sg[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                                 {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    for (int k = 0; k < 8; k++)
        test1(V3(sg[k][0] > 0 ? p.x : -p.x, sg[k][1] > 0 ? p.y : -p.y, sg[k][2] > 0 ? p.z : -p.z));
    double s;
    V3 v;
    if (-p.x <= cB.x && cB.x <= p.x) {
        if (cB.y >= p.y && cB.z >= p.z) { v = V3(0, cB.y - p.y, cB.z - p.z); s = vlength(v); s -= r; test2(s, cB.x, p.y, p.z, v.x, v.y, v.z); }
        else if (cB.y <= -p.y && cB.z >= p.z) { v = V3(0, cB.y + p.y, cB.z - p.z); s = vlength(v); s -= r; test2(s, cB.x, -p.y, p.z, v.x, v.y, v.z); }
        else if (cB.y >= p.y && cB.z <= -p.z) { v = V3(0, cB.y - p.y, cB.z + p.z); s = vlength(v); s -= r; test2(s, cB.x, p.y, -p.z, v.x, v.y, v.z); }
        else if (cB.y <= -p.y && cB.z <= -p.z) { v = V3(0, cB.y + p.y, cB.z + p.z); s = vlength(v); s -= r; test2(s, cB.x, -p.y, -p.z, v.x, v.y, v.z); }
    }
    if (-p.y <= cB.y && cB.y <= p.y) {
        if (cB.x >= p.x && cB.z >= p.z) { v = V3(cB.x - p.x, 0, cB.z - p.z); s = vlength(v); s -= r; test2(s, p.x, cB.y, p.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.z >= p.z) { v = V3(cB.x + p.x, 0, cB.z - p.z); s = vlength(v); s -= r; test2(s, -p.x, cB.y, p.z, v.x, v.y, v.z); }
        else if (cB.x >= p.x && cB.z <= -p.z) { v = V3(cB.x - p.x, 0, cB.z + p.z); s = vlength(v); s -= r; test2(s, p.x, cB.y, -p.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.z <= -p.z) { v = V3(cB.x + p.x, 0, cB.z + p.z); s = vlength(v); s -= r; test2(s, -p.x, cB.y, -p.z, v.x, v.y, v.z); }
    }
    if (-p.z <= cB.z && cB.z <= p.z) {
        if (cB.x >= p.x && cB.y >= p.y) { v = V3(cB.x - p.x, cB.y - p.y, 0); s = vlength(v); s -= r; test2(s, p.x, p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.y >= p.y) { v = V3(cB.x + p.x, cB.y - p.y, 0); s = vlength(v); s -= r; test2(s, -p.x, p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x >= p.x && cB.y <= -p.y) { v = V3(cB.x - p.x, cB.y + p.y, 0); s = vlength(v); s -= r; test2(s, p.x, -p.y, cB.z, v.x, v.y, v.z); }
        else if (cB.x <= -p.x && cB.y <= -p.y) { v = V3(cB.x + p.x, cB.y + p.y, 0); s = vlength(v); s -= r; test2(s, -p.x, -p.y, cB.z, v.x, v.y, v.z); }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.y <= cB.y && cB.y <= p.y) {
        if (cB.z > 0) { s = cB.z - p.z - r; test2(s, cB.x, cB.y, p.z, 0, 0, 1); }
        else { s = -p.z - cB.z - r; test2(s, cB.x, cB.y, -p.z, 0, 0, -1); }
    }
    if (-p.x <= cB.x && cB.x <= p.x && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.y > 0) { s = cB.y - p.y - r; test2(s, cB.x, p.y, cB.z, 0, 1, 0); }
        else { s = -p.y - cB.y - r; test2(s, cB.x, -p.y, cB.z, 0, -1, 0); }
    }
    if (-p.y <= cB.y && cB.y <= p.y && -p.z <= cB.z && cB.z <= p.z) {
        if (cB.x > 0) { s = cB.x - p.x - r; test2(s, p.x, cB.y, cB.z, 1, 0, 0); }
        else { s = -p.x - cB.x - r; test2(s, -p.x, cB.y, cB.z, -1, 0, 0); }
    }
    if (depth != 1) {
        RT T = box->T();
        pos = rt_point(T, pos);
        nrm = rt_vec(T, nrm);
        vnormalize(nrm);
        emit(box, sph, pos, nrm, AM_BV_NULL, AM_BV_NULL, 0, depth);
    }
}

// ---------------------------------------------------------------------------
// BoxBox.dBoxBox (collision/BoxBox.java:433-859; ODE's separating-axis box
// test).  Operation order kept: TST1 with tinyOffset 1e-5 (:291-310), TST2
// with fudgeFactor 1.05 (:313-336), dLineClosestApproach (:366-383),
// intersectRectQuad (:140-209).  The cull branch is unreachable (maxc=0xffff).
static inline double gcomp(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

static int clipRectQuad(const double h[2], const double quad[8], double ret[16]) {
    double buffer[16];
    const double* q = quad;
    double* r = ret;
    int nq = 4, nr = 0;
    for (int dir = 0; dir <= 1; dir++) {
        for (int sign = -1; sign <= 1; sign += 2) {
            int pq = 0, pr = 0;
            nr = 0;
            for (int i = nq; i > 0; i--) {
                if ((double)sign * q[pq + dir] < h[dir]) {
                    r[pr] = q[pq];
                    r[pr + 1] = q[pq + 1];
                    pr += 2;
                    nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                int nx = (i > 1) ? pq + 2 : 0;
                if (((double)sign * q[pq + dir] < h[dir]) ^ ((double)sign * q[nx + dir] < h[dir])) {
                    r[pr + 1 - dir] = q[pq + 1 - dir] +
                                      (q[nx + 1 - dir] - q[pq + 1 - dir]) / (q[nx + dir] - q[pq + dir]) *
                                          ((double)sign * h[dir] - q[pq + dir]);
                    r[pr + dir] = (double)sign * h[dir];
                    pr += 2;
                    nr++;
                    if (nr & 8) { q = r; goto done; }
                }
                pq += 2;
            }
            q = r;
            r = (q == ret) ? buffer : ret;
            nq = nr;
        }
    }
done:
    if (q != ret) std::memcpy(ret, q, sizeof(double) * 2 * nr);
    return nr;
}

void World::boxBox(Body* b1, Body* b2) {
    const V3& p1 = b1->x;
    const V3& p2 = b2->x;
    const M3& R1 = b1->theta;
    const M3& R2 = b2->theta;
    V3 p = vsub(p2, p1);
    if (vlength(p) > b1->radius + b2->radius) return;
    V3 pp = mtxv(R1, p);
    V3 A = vscale(0.5, b1->size);
    V3 B = vscale(0.5, b2->size);
    auto d44 = [](const M3& a, int o1, const M3& b, int o2) { return vdot(a.col(o1), b.col(o2)); };
    double R11 = d44(R1, 0, R2, 0), R12 = d44(R1, 0, R2, 1), R13 = d44(R1, 0, R2, 2);
    double R21 = d44(R1, 1, R2, 0), R22 = d44(R1, 1, R2, 1), R23 = d44(R1, 1, R2, 2);
    double R31 = d44(R1, 2, R2, 0), R32 = d44(R1, 2, R2, 1), R33 = d44(R1, 2, R2, 2);
    double Q11 = std::fabs(R11), Q12 = std::fabs(R12), Q13 = std::fabs(R13);
    double Q21 = std::fabs(R21), Q22 = std::fabs(R22), Q23 = std::fabs(R23);
    double Q31 = std::fabs(R31), Q32 = std::fabs(R32), Q33 = std::fabs(R33);

    double s = -INFINITY;
    bool invert = false;
    int code = 0;
    const M3* normalM = nullptr;
    int normalCol = 0;
    V3 normalC;
    const double tinyOffset = 1e-5, fudge = 1.05;
    auto tst1 = [&](double e1, double e2, const M3* M, int col, int cc) {
        double s2 = std::fabs(e1) - e2;
        if (s2 > 0) return false;
        if (s2 > s + tinyOffset) { s = s2; normalM = M; normalCol = col; invert = e1 < 0; code = cc; }
        return true;
    };
    auto tst2 = [&](double e1, double e2, double n1, double n2, double n3, int cc) {
        double s2 = std::fabs(e1) - e2;
        if (s2 > 0) return false;
        double l = std::sqrt(n1 * n1 + n2 * n2 + n3 * n3);
        if (l > 0) {
            s2 /= l;
            if (s2 * fudge > s) { s = s2; normalM = nullptr; normalCol = 0; normalC = V3(n1 / l, n2 / l, n3 / l); invert = e1 < 0; code = cc; }
        }
        return true;
    };
    if (!tst1(pp.x, A.x + B.x * Q11 + B.y * Q12 + B.z * Q13, &R1, 0, 1)) return;
    if (!tst1(pp.y, A.y + B.x * Q21 + B.y * Q22 + B.z * Q23, &R1, 1, 2)) return;
    if (!tst1(pp.z, A.z + B.x * Q31 + B.y * Q32 + B.z * Q33, &R1, 2, 3)) return;
    if (!tst1(vdot(R2.col(0), p), A.x * Q11 + A.y * Q21 + A.z * Q31 + B.x, &R2, 0, 4)) return;
    if (!tst1(vdot(R2.col(1), p), A.x * Q12 + A.y * Q22 + A.z * Q32 + B.y, &R2, 1, 5)) return;
    if (!tst1(vdot(R2.col(2), p), A.x * Q13 + A.y * Q23 + A.z * Q33 + B.z, &R2, 2, 6)) return;
    if (!tst2(pp.z * R21 - pp.y * R31, A.y * Q31 + A.z * Q21 + B.y * Q13 + B.z * Q12, 0, -R31, R21, 7)) return;
    if (!tst2(pp.z * R22 - pp.y * R32, A.y * Q32 + A.z * Q22 + B.x * Q13 + B.z * Q11, 0, -R32, R22, 8)) return;
    if (!tst2(pp.z * R23 - pp.y * R33, A.y * Q33 + A.z * Q23 + B.x * Q12 + B.y * Q11, 0, -R33, R23, 9)) return;
    if (!tst2(pp.x * R31 - pp.z * R11, A.x * Q31 + A.z * Q11 + B.y * Q23 + B.z * Q22, R31, 0, -R11, 10)) return;
    if (!tst2(pp.x * R32 - pp.z * R12, A.x * Q32 + A.z * Q12 + B.x * Q23 + B.z * Q21, R32, 0, -R12, 11)) return;
    if (!tst2(pp.x * R33 - pp.z * R13, A.x * Q33 + A.z * Q13 + B.x * Q22 + B.y * Q21, R33, 0, -R13, 12)) return;
    if (!tst2(pp.y * R11 - pp.x * R21, A.x * Q21 + A.y * Q11 + B.y * Q33 + B.z * Q32, -R21, R11, 0, 13)) return;
    if (!tst2(pp.y * R12 - pp.x * R22, A.x * Q22 + A.y * Q12 + B.x * Q33 + B.z * Q31, -R22, R12, 0, 14)) return;
    if (!tst2(pp.y * R13 - pp.x * R23, A.x * Q23 + A.y * Q13 + B.x * Q32 + B.y * Q31, -R23, R13, 0, 15)) return;
    if (code == 0) return;

    V3 normal = normalM ? normalM->col(normalCol) : mxv(R1, normalC);
    if (invert) vscale_ip(normal, -1);
    double depth = -s;
    int info = 0;

    if (code > 6) {  // edge-edge
        V3 pa = p1;
        for (int j = 0; j < 3; j++) {
            double sign = (vdot(normal, R1.col(j)) > 0) ? 1.0 : -1.0;
            pa.x += sign * gcomp(A, j) * R1.get(0, j);
            pa.y += sign * gcomp(A, j) * R1.get(1, j);
            pa.z += sign * gcomp(A, j) * R1.get(2, j);
        }
        V3 pb = p2;
        for (int j = 0; j < 3; j++) {
            double sign = (vdot(normal, R2.col(j)) > 0) ? -1.0 : 1.0;
            pb.x += sign * gcomp(B, j) * R2.get(0, j);
            pb.y += sign * gcomp(B, j) * R2.get(1, j);
            pb.z += sign * gcomp(B, j) * R2.get(2, j);
        }
        V3 ua = R1.col((code - 7) / 3);
        V3 ub = R2.col((code - 7) % 3);
        // dLineClosestApproach
        V3 q = vsub(pb, pa);
        double uaub = vdot(ua, ub);
        double q1 = vdot(ua, q);
        double q2 = -vdot(ub, q);
        double d = 1 - uaub * uaub;
        double alpha, beta;
        if (d <= 0.0001) { alpha = 0; beta = 0; }
        else { d = 1.0 / d; alpha = (q1 + uaub * q2) * d; beta = (uaub * q1 + q2) * d; }
        pa = vscaleadd(alpha, ua, pa);
        pb = vscaleadd(beta, ub, pb);
        V3 pos = vadd(pa, pb);
        vscale_ip(pos, 0.5);
        emit(b1, b2, pos, normal, AM_BV_NULL, AM_BV_NULL, info++, -depth);
        return;
    }
    // face-something: reference face a, incident face b
    const M3 *Ra, *Rb;
    const V3 *pa, *pb, *Sa, *Sb;
    if (code <= 3) { Ra = &R1; Rb = &R2; pa = &p1; pb = &p2; Sa = &A; Sb = &B; }
    else { Ra = &R2; Rb = &R1; pa = &p2; pb = &p1; Sa = &B; Sb = &A; }
    V3 normal2 = (code <= 3) ? normal : vscale(-1, normal);
    V3 nr = mtxv(*Rb, normal2);
    V3 anr(std::fabs(nr.x), std::fabs(nr.y), std::fabs(nr.z));
    int lanr, a1, a2;
    if (anr.y > anr.x) {
        if (anr.y > anr.z) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr.x > anr.z) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    V3 center;
    if (gcomp(nr, lanr) < 0) {
        for (int i = 0; i < 3; i++) center[i] = gcomp(*pb, i) - gcomp(*pa, i) + gcomp(*Sb, lanr) * Rb->get(i, lanr);
    } else {
        for (int i = 0; i < 3; i++) center[i] = gcomp(*pb, i) - gcomp(*pa, i) - gcomp(*Sb, lanr) * Rb->get(i, lanr);
    }
    int codeN, code1, code2;
    codeN = (code <= 3) ? code - 1 : code - 4;
    if (codeN == 0) { code1 = 1; code2 = 2; }
    else if (codeN == 1) { code1 = 0; code2 = 2; }
    else { code1 = 0; code2 = 1; }
    double c1 = vdot(center, Ra->col(code1));
    double c2 = vdot(center, Ra->col(code2));
    double m11 = d44(*Ra, code1, *Rb, a1);
    double m12 = d44(*Ra, code1, *Rb, a2);
    double m21 = d44(*Ra, code2, *Rb, a1);
    double m22 = d44(*Ra, code2, *Rb, a2);
    double quad[8];
    {
        double k1 = m11 * gcomp(*Sb, a1);
        double k2 = m21 * gcomp(*Sb, a1);
        double k3 = m12 * gcomp(*Sb, a2);
        double k4 = m22 * gcomp(*Sb, a2);
        quad[0] = c1 - k1 - k3;
        quad[1] = c2 - k2 - k4;
        quad[2] = c1 - k1 + k3;
        quad[3] = c2 - k2 + k4;
        quad[4] = c1 + k1 + k3;
        quad[5] = c2 + k2 + k4;
        quad[6] = c1 + k1 - k3;
        quad[7] = c2 + k2 - k4;
    }
    double rect[2] = {gcomp(*Sa, code1), gcomp(*Sa, code2)};
    double ret[16];
    int n = clipRectQuad(rect, quad, ret);
    if (n < 1) return;
    double det1 = 1.0 / (m11 * m22 - m12 * m21);
    m11 *= det1; m12 *= det1; m21 *= det1; m22 *= det1;
    double point[24], dep[8];
    int cnum = 0;
    for (int j = 0; j < n; j++) {
        double k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        double k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (int i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb->get(i, a1) + k2 * Rb->get(i, a2);
        dep[cnum] = gcomp(*Sa, codeN) - (normal2.x * point[cnum * 3] + normal2.y * point[cnum * 3 + 1] + normal2.z * point[cnum * 3 + 2]);
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return;
    for (int j = 0; j < cnum; j++) {
        V3 pos;
        for (int i = 0; i < 3; i++) pos[i] = point[j * 3 + i] + gcomp(*pa, i);
        emit(b1, b2, pos, normal, AM_BV_NULL, AM_BV_NULL, info++, -dep[j]);
    }
}

// ---------------------------------------------------------------------------
// Sphere trees: collideSphereTreeAndPlane, collideBoxAndSphereTree,
// collideSphereTrees, processCollision (CollisionProcessor.java:793-826,
// 837-850, 975-1009, 1036-1056).  World centres are refreshed once per step
// before the broad phase, which gives the same values as the visitID refresh.
void World::treePlane(int ni, Body* b, Body* plane) {
    Node& nd = nodes[ni];
    const V3& c = nd.cW;
    const V3& n = plane->pn;
    double d = n.x * c.x + n.y * c.y + n.z * c.z + plane->pd - nd.r;
    if (d < 0) {
        if (nd.child0 < 0) {
            V3 t = vsub(c, plane->pp);
            double val = vdot(t, plane->pn);
            t = vscale(val, plane->pn);
            V3 cw = vsub(c, t);
            V3 nrm = vscale(-1, plane->pn);
            emit(b, plane, cw, nrm, ni, AM_BV_PLANE(plane->id), 0, d);
        } else {
            for (int k = 0; k < nd.nchild; k++) treePlane(nd.child0 + k, b, plane);
        }
    }
}

void World::boxTree(int ni, Body* box, Body* tree) {
    Node& nd = nodes[ni];
    if (!boxSphereTest(box, nd.cW, nd.r)) return;
    if (nd.child0 >= 0) {
        for (int k = 0; k < nd.nchild; k++) boxTree(nd.child0 + k, box, tree);
    } else {
        boxSphere(box, tree, nd.cW, nd.r);
    }
}

void World::treeTree(int i1, int i2, Body* b1, Body* b2) {
    Node& n1 = nodes[i1];
    Node& n2 = nodes[i2];
    if (pdist2(n1.cW, n2.cW) < (n1.r + n2.r) * (n1.r + n2.r)) {
        bool l1 = n1.child0 < 0, l2 = n2.child0 < 0;
        if (l1 && l2) {
            double distance = pdist(n1.cW, n2.cW);
            double dbc = n2.r + n1.r;
            if (distance < dbc) {
                double alpha = (n1.r - n2.r + distance) / (2 * distance);
                V3 cw = vinterp(n1.cW, n2.cW, alpha);
                V3 nrm = vsub(n2.cW, n1.cW);
                vnormalize(nrm);
                emit(b1, b2, cw, nrm, i1, i2, 0, distance - dbc);
            }
        } else if (l1) {
            for (int k = 0; k < n2.nchild; k++) treeTree(i1, n2.child0 + k, b1, b2);
        } else if (l2) {
            for (int k = 0; k < n1.nchild; k++) treeTree(n1.child0 + k, i2, b1, b2);
        } else if (n1.r <= n2.r) {
            for (int k = 0; k < n2.nchild; k++) treeTree(i1, n2.child0 + k, b1, b2);
        } else {
            for (int k = 0; k < n1.nchild; k++) treeTree(n1.child0 + k, i2, b1, b2);
        }
    }
}

// CollisionProcessor.narrowPhase / narrowPhaseCollection (brute force)
// (CollisionProcessor.java:707-791)
void World::narrowPhase(Body* b1, Body* b2) {
    if (b1->isCollection || b2->isCollection) {
        if (b1->isCollection) { for (Body* b : b1->bodies) narrowPhase(b, b2); }
        else { for (Body* b : b2->bodies) narrowPhase(b1, b); }
        return;
    }
    if (b1->type == ORC_COMPOSITE) {           // CollisionProcessor.java:711-716
        for (Body* b : b1->subs) narrowPhase(b, b2);
        return;
    }
    if (b2->type == ORC_COMPOSITE) {           // :717-722
        for (Body* b : b2->subs) narrowPhase(b1, b);
        return;
    }
    if (b1->type == AM_PLANE) {
        if (b2->type == AM_PLANE) return;
        if (b2->type == AM_BOX) boxPlane(b2, b1);
        else treePlane(b2->root, b2, b1);
    } else if (b1->type == AM_BOX) {
        if (b2->type == AM_PLANE) boxPlane(b1, b2);
        else if (b2->type == AM_BOX) boxBox(b1, b2);
        else boxTree(b2->root, b1, b2);
    } else {
        if (b2->type == AM_PLANE) treePlane(b1->root, b1, b2);
        else if (b2->type == AM_BOX) boxTree(b1->root, b2, b1);
        else treeTree(b1->root, b2->root, b1, b2);
    }
}

// CollisionProcessor.collisionDetection + broadPhase (CollisionProcessor.java:91-102, 683-697)
void World::collisionDetection() {
    contacts.clear();
    cur ^= 1;
    pool[cur].clear();
    updateCompositeSubs();
    for (auto& n : nodes) n.cW = rt_point(n.body->T(), n.cB);   // BVSphere.updatecW
    size_t N = bodies.size();
    for (size_t i = 0; i + 1 < N; i++) {
        Body* b1 = bodies[i];
        for (size_t j = i + 1; j < N; j++) {
            Body* b2 = bodies[j];
            if (b1->pinned && b2->pinned) continue;
            if ((b1->pinned && b2->sleeping) || (b2->pinned && b1->sleeping)) continue;
            narrowPhase(b1, b2);
        }
    }
    if (contacts.empty()) last.clear();
}

// CollisionProcessor.updateContactsMap (CollisionProcessor.java:443-448)
void World::updateContactsMap() {
    last.clear();
    for (Contact* c : contacts) last[ckey(c, c->info)] = c;
}

// ---------------------------------------------------------------------------
// Body-pair contacts: updateBodyPairContacts, storeInBodyPairContacts,
// removeEmptyBodyPairContacts, clearBodyPairContacts
// (CollisionProcessor.java:145-226); BodyPairContact.checkExists /
// addToBodyLists / addToBodyListsParent / removeFrom* (BodyPairContact.java:54-348)
static uint64_t pairKey(const Body* a, const Body* b) {
    uint32_t x = (uint32_t)std::min(a->id, b->id), y = (uint32_t)std::max(a->id, b->id);
    return ((uint64_t)x << 32) | y;
}
static void addToBodyLists(BPC* p) { p->body1->bpcs.add(p); p->body2->bpcs.add(p); }
static void addToBodyListsParent(BPC* p) {
    if (p->body1->parent) p->body1->parent->bpcs.add(p);
    if (p->body2->parent) p->body2->parent->bpcs.add(p);
}
static void removeFromBodyLists(BPC* p) { p->body1->bpcs.remove(p); p->body2->bpcs.remove(p); }
static void removeFromBodyListsParent(BPC* p) {
    if (p->body1->parent) p->body1->parent->bpcs.remove(p);
    if (p->body2->parent) p->body2->parent->bpcs.remove(p);
}

void World::updateBPCsForContact(Contact* c) {
    if (c->body1->pinned && c->body2->pinned) return;
    uint64_t k = pairKey(c->body1, c->body2);
    BPC* p = nullptr;
    auto it = bpcIndex.find(k);
    if (it != bpcIndex.end() && bodyPairContacts.contains(it->second)) {
        p = it->second;
    } else {   // index stale: search the set as BodyPairContact.checkExists does
        for (BPC* q : bodyPairContacts.v)
            if ((q->body1 == c->body1 && q->body2 == c->body2) || (q->body1 == c->body2 && q->body2 == c->body1)) { p = q; bpcIndex[k] = q; break; }
    }
    if (!p) {
        bpcStore.emplace_back();
        p = &bpcStore.back();
        p->body1 = c->body1;
        p->body2 = c->body2;
        bodyPairContacts.add(p);
        bpcIndex[k] = p;
    }
    addToBodyLists(p);
    addToBodyListsParent(p);
    p->contactList.push_back(c);
}

void World::removeEmptyBodyPairContacts() {
    std::vector<BPC*> keep;
    bool updated = false;
    for (BPC* p : bodyPairContacts.v) {
        if (!p->contactList.empty()) keep.push_back(p);
        else { removeFromBodyLists(p); removeFromBodyListsParent(p); updated = true; }
    }
    if (updated) {
        bodyPairContacts.clear();
        for (BPC* p : keep) bodyPairContacts.add(p);
    }
}

void World::updateBodyPairContacts() {
    for (BPC* p : bodyPairContacts.v) { p->checked = false; p->contactList.clear(); }
    for (Body* b : bodies)
        if (b->isCollection)
            for (BPC* p : b->bpcs.v) p->checked = false;
    for (Contact* c : contacts) updateBPCsForContact(c);
    removeEmptyBodyPairContacts();
}

void World::clearBodyPairContacts() {
    for (BPC* p : bodyPairContacts.v) {
        std::vector<Contact*> keep;
        for (Contact* c : p->contactList)
            if (std::fabs(c->l0) > 1e-14) keep.push_back(c);
        p->contactList = keep;
    }
    removeEmptyBodyPairContacts();
}

// ---------------------------------------------------------------------------
// CollisionProcessor.warmStart / vanillaWarmStart (CollisionProcessor.java:481-665)
static void takeOld(Contact* c, Contact* o) {
    c->fresh = false;
    c->l0 = o->l0; c->l1 = o->l1; c->l2 = o->l2;
    c->l0w = o->l0; c->l1w = o->l1; c->l2w = o->l2;
}

void World::warmStart() {
    auto vanilla = [&](Contact* c) {   // vanillaWarmStart (:646-665)
        auto it = last.find(ckey(c, c->info));
        if (it != last.end()) { takeOld(c, it->second); c->prevCv = it->second->cv; }
        else c->fresh = true;
    };
    // RigidBodyGeomBox or RigidBodyGeomComposite (:488-493)
    auto boxy = [](const Body* b) { return (b->type == AM_BOX || b->type == ORC_COMPOSITE) && !b->isCollection; };
    auto nonBoxSub = [&](int csb) { return csb >= 0 && subStore[csb - ORC_SUB_ID0].type != AM_BOX; };
    for (BPC* bpc : bodyPairContacts.v) {
        if (bpc->inCollection) continue;
        if (boxy(bpc->body1) && boxy(bpc->body2)) {
            for (Contact* c : bpc->contactList) {
                // a composite's non-box sub-body takes the plain warm start; for
                // csb2 the reference does not skip the box-box search afterwards
                // (:494-503)
                if (nonBoxSub(c->csb1)) { vanilla(c); continue; }
                if (nonBoxSub(c->csb2)) vanilla(c);
                V3 pNew = rt_point(c->body1->T(), c->cB1);
                auto look = [&](int info) -> Contact* {
                    auto it = last.find(ckey(c, info));
                    return it == last.end() ? nullptr : it->second;
                };
                Contact* old = look(c->info);
                if (old) {
                    V3 pOld = rt_point(old->body1->T(), old->cB1);
                    double dist = pdist(pNew, pOld);
                    if (dist > 0.05) {
                        int myInfo = c->info;
                        double best = dist;
                        Contact* bestOld = old;
                        for (int info = 0; info < 9; info++) {
                            if (info == myInfo) continue;
                            Contact* o2 = look(info);
                            if (!o2) break;
                            pOld = rt_point(o2->body1->T(), o2->cB1);
                            double d2 = pdist(pNew, pOld);
                            if (d2 < best) { best = d2; bestOld = o2; }
                        }
                        old = bestOld;
                        dist = best;
                    }
                    if (dist < 0.05) {
                        takeOld(c, old);
                        old->l0 = old->l1 = old->l2 = 0;
                        c->prevCv = old->cv;
                    } else {
                        c->fresh = true;
                    }
                } else {
                    double best = 1.79769313486231570e308;
                    int bestInfo = -1;
                    Contact* bestOld = nullptr;
                    for (int info = 0; info < 9; info++) {
                        Contact* o2 = look(info);
                        if (!o2) break;
                        V3 pOld = rt_point(o2->body1->T(), o2->cB1);
                        double d2 = pdist(pNew, pOld);
                        if (d2 < best) { best = d2; bestInfo = info; bestOld = o2; }
                    }
                    if (bestInfo != -1) {
                        if (best < 0.05) {
                            takeOld(c, bestOld);
                            bestOld->l0 = bestOld->l1 = bestOld->l2 = 0;
                            c->prevCv = bestOld->cv;
                        }
                    } else {
                        c->fresh = true;
                    }
                }
            }
        } else {
            for (Contact* c : bpc->contactList) vanilla(c);
        }
    }
}

void World::redoWarmStart() {  // CollisionProcessor.java:453-459
    for (Contact* c : contacts) { c->l0 = c->l0w; c->l1 = c->l1w; c->l2 = c->l2w; }
}

// ---------------------------------------------------------------------------
// PGS.solve, updateDeltaVwithLambdai, confidentWarmStart (PGS.java:73-256);
// Contact.computeB / computeJMinvJt / getJdv / updateContactState
// (Contact.java:279-398)
static inline Body* solveBody(Body* b, bool inColl) { return (b->parent && !inColl) ? b->parent : b; }

static void computeB(Contact* c, double dt, double fb, bool inColl, bool restOv, double restVal) {
    Body* b1 = solveBody(c->body1, inColl);
    Body* b2 = solveBody(c->body2, inColl);
    double restitution = (c->body1->restitution + c->body2->restitution) / 2.;
    if (restOv) restitution = restVal;
    double bn = 0, bt1 = 0, bt2 = 0;
    V3 t = vscaleadd(b1->minv * dt, b1->force, b1->v);
    bn += vdot(t, c->jna_v); bt1 += vdot(t, c->jt1a_v); bt2 += vdot(t, c->jt2a_v);
    t = mxv(b1->jinv, b1->torque);
    vscale_ip(t, dt);
    t = vadd(t, b1->omega);
    bn += vdot(t, c->jna_w); bt1 += vdot(t, c->jt1a_w); bt2 += vdot(t, c->jt2a_w);
    double bb = vdot(b1->v, c->jna_v) + vdot(b1->omega, c->jna_w);
    bb *= restitution;
    bn += bb;
    t = vscaleadd(b2->minv * dt, b2->force, b2->v);
    bn += vdot(t, c->jnb_v); bt1 += vdot(t, c->jt1b_v); bt2 += vdot(t, c->jt2b_v);
    t = mxv(b2->jinv, b2->torque);
    vscale_ip(t, dt);
    t = vadd(t, b2->omega);
    bn += vdot(t, c->jnb_w); bt1 += vdot(t, c->jt1b_w); bt2 += vdot(t, c->jt2b_w);
    bb = vdot(b2->v, c->jnb_v) + vdot(b2->omega, c->jnb_w);
    bb *= restitution;
    bn += bb;
    bn += fb * c->cv;
    c->bn = bn; c->bt1 = bt1; c->bt2 = bt2;
}

static void computeJMinvJt(Contact* c, bool inColl) {
    Body* b1 = solveBody(c->body1, inColl);
    Body* b2 = solveBody(c->body2, inColl);
    V3 t1 = mxv(b1->jinv, c->jna_w), t2 = mxv(b2->jinv, c->jnb_w);
    c->D00 = b1->minv * vdot(c->jna_v, c->jna_v) + vdot(c->jna_w, t1) + b2->minv * vdot(c->jnb_v, c->jnb_v) + vdot(c->jnb_w, t2);
    t1 = mxv(b1->jinv, c->jt1a_w); t2 = mxv(b2->jinv, c->jt1b_w);
    c->D11 = b1->minv * vdot(c->jt1a_v, c->jt1a_v) + vdot(c->jt1a_w, t1) + b2->minv * vdot(c->jt1b_v, c->jt1b_v) + vdot(c->jt1b_w, t2);
    t1 = mxv(b1->jinv, c->jt2a_w); t2 = mxv(b2->jinv, c->jt2b_w);
    c->D22 = b1->minv * vdot(c->jt2a_v, c->jt2a_v) + vdot(c->jt2a_w, t1) + b2->minv * vdot(c->jt2b_v, c->jt2b_v) + vdot(c->jt2b_w, t2);
}

static inline void rowJ(const Contact* c, int i, const V3*& av, const V3*& aw, const V3*& bv, const V3*& bw) {
    if (i == 0) { av = &c->jna_v; aw = &c->jna_w; bv = &c->jnb_v; bw = &c->jnb_w; }
    else if (i == 1) { av = &c->jt1a_v; aw = &c->jt1a_w; bv = &c->jt1b_v; bw = &c->jt1b_w; }
    else { av = &c->jt2a_v; aw = &c->jt2a_w; bv = &c->jt2b_v; bw = &c->jt2b_w; }
}

static double getJdv(const Contact* c, bool inColl, int i) {
    Body* b1 = solveBody(c->body1, inColl);
    Body* b2 = solveBody(c->body2, inColl);
    const V3 *av, *aw, *bv, *bw;
    rowJ(c, i, av, aw, bv, bw);
    return (vdot(*av, b1->dvv) + vdot(*aw, b1->dvw)) + (vdot(*bv, b2->dvv) + vdot(*bw, b2->dvw));
}

static void updateDeltaV(Contact* c, bool inColl, double lambda, int i) {
    Body* b1 = solveBody(c->body1, inColl);
    Body* b2 = solveBody(c->body2, inColl);
    const V3 *av, *aw, *bv, *bw;
    rowJ(c, i, av, aw, bv, bw);
    b1->dvv = vscaleadd(b1->minv * lambda, *av, b1->dvv);
    V3 t = mxv(b1->jinv, *aw);
    b1->dvw = vscaleadd(lambda, t, b1->dvw);
    b2->dvv = vscaleadd(b2->minv * lambda, *bv, b2->dvv);
    t = mxv(b2->jinv, *bw);
    b2->dvw = vscaleadd(lambda, t, b2->dvw);
}

void World::pgs(std::vector<Contact*>& list, double dt, bool inColl, int iters, double fb, double comp, bool early) {
    if (list.empty()) return;
    for (Contact* c : list) {  // confidentWarmStart
        updateDeltaV(c, inColl, c->l0, 0);
        updateDeltaV(c, inColl, c->l1, 1);
        updateDeltaV(c, inColl, c->l2, 2);
    }
    for (Contact* c : list) {
        computeB(c, dt, fb, inColl, P.restitution_override != 0, P.restitution);
        computeJMinvJt(c, inColl);
    }
    const double omega = P.omega;
    int iter = iters;
    int done = 0;
    double change = 0;
    while (iter > 0) {
        double mx = 0;
        for (Contact* c : list) {
            double Jdvn = getJdv(c, inColl, 0);
            double prev = c->l0;
            c->l0 = (c->D00 * c->l0 - omega * (c->bn + Jdvn)) / (c->D00 + comp);
            c->l0 = jmax(0.0, c->l0);
            double diff = c->l0 - prev;
            updateDeltaV(c, inColl, diff, 0);
            mx = jmax(mx, std::fabs(diff));
            double mu;
            if (P.friction_override) mu = P.friction;
            else {
                double f1 = c->body1->friction, f2 = c->body2->friction;
                if (f1 < 0.2 || f2 < 0.2) mu = jmin(f1, f2);
                else if (f1 > 1. || f2 > 1.) mu = jmax(f1, f2);
                else mu = (f1 + f2) / 2.;
            }
            double Jdv1 = getJdv(c, inColl, 1);
            prev = c->l1;
            c->l1 = (c->D11 * c->l1 - omega * (c->bt1 + Jdv1)) / (c->D11 + comp);
            double lim = mu * c->l0;
            c->l1 = jmax(c->l1, -lim);
            c->l1 = jmin(c->l1, lim);
            diff = c->l1 - prev;
            updateDeltaV(c, inColl, diff, 1);
            mx = jmax(mx, std::fabs(diff));
            double Jdv2 = getJdv(c, inColl, 2);
            prev = c->l2;
            c->l2 = (c->D22 * c->l2 - omega * (c->bt2 + Jdv2)) / (c->D22 + comp);
            lim = mu * c->l0;
            c->l2 = jmax(c->l2, -lim);
            c->l2 = jmin(c->l2, lim);
            diff = c->l2 - prev;
            updateDeltaV(c, inColl, diff, 2);
            mx = jmax(mx, std::fabs(diff));
            if (iter == 1) {  // Contact.updateContactState
                c->w1 = c->bt1 + getJdv(c, inColl, 1);
                c->w2 = c->bt2 + getJdv(c, inColl, 2);
                if (std::fabs(c->l0) <= 1e-14) c->state = BROKEN;
                else if (std::fabs(c->w1) > P.sliding_threshold) c->state = ONEDGE;
                else if (std::fabs(c->w2) > P.sliding_threshold) c->state = ONEDGE;
                else c->state = CLEAR;
            }
        }
        iter--;
        done++;
        change = mx;
        if (early && mx < P.tolerance) break;
        if (!inColl && resTarget > 0 && resCheck > 0 && (done % resCheck == 0 || iter == 0) &&
            relResidual(list, comp) <= resTarget)
            break;
    }
    if (!inColl) { stats.sweeps = done; stats.last_change = change; }
}

// max_i |l_i - proj(l_i - w_i / (D_ii + c))| / max(1, max |l|) with
// w = b + J dv + c l: the natural-map residual of the full solve's LCP
double World::relResidual(std::vector<Contact*>& list, double comp) {
    double rmax = 0, lmax = 0;
    for (Contact* c : list) {
        double mu;
        if (P.friction_override) mu = P.friction;
        else {
            double f1 = c->body1->friction, f2 = c->body2->friction;
            if (f1 < 0.2 || f2 < 0.2) mu = jmin(f1, f2);
            else if (f1 > 1. || f2 > 1.) mu = jmax(f1, f2);
            else mu = (f1 + f2) / 2.;
        }
        const double l[3] = {c->l0, c->l1, c->l2};
        const double b[3] = {c->bn, c->bt1, c->bt2};
        const double D[3] = {c->D00, c->D11, c->D22};
        for (int i = 0; i < 3; i++) {
            double w = b[i] + getJdv(c, false, i) + comp * l[i];
            double z = l[i] - w / (D[i] + comp);
            if (i == 0) z = std::max(z, 0.0);
            else z = std::min(std::max(z, -mu * l[0]), mu * l[0]);
            rmax = std::max(rmax, std::fabs(l[i] - z));
            lmax = std::max(lmax, std::fabs(l[i]));
        }
    }
    return rmax / std::max(1.0, lmax);
}

// CollisionProcessor.solveLCP (CollisionProcessor.java:108-137)
void World::solveLCP(double dt) {
    if (contacts.empty()) { stats.sweeps = 0; stats.last_change = 0; return; }
    double comp = P.enable_compliance ? P.compliance : 0.;
    for (Contact* c : contacts)   // updateJacobiansThatNeedUpdating(contacts, false)
        if (c->body1->parent || c->body2->parent) recomputeJacobian(c, false);
    pgs(contacts, dt, false, P.iterations, P.feedback_stiffness, comp, true);
}

// ---------------------------------------------------------------------------
// Single sweep inside collections: updateInCollections, getOrganizedContacts,
// getNextLayer (CollisionProcessor.java:232-441)
void World::getNextLayer(std::vector<BPC*>& layer, std::vector<BPC*>& ordered) {
    std::vector<BPC*> next;
    for (BPC* p : layer)
        for (int i = 0; i < 2; i++) {
            Body* b = p->getBody(i);
            for (BPC* o : b->bpcs.v)
                if (!o->checked) { next.push_back(o); o->checked = true; }
        }
    if (!next.empty()) {
        for (BPC* p : next) ordered.push_back(p);
        getNextLayer(next, ordered);
    }
}

void World::getOrganizedContacts(std::vector<Contact*>& out) {
    std::vector<BPC*> ordered;
    for (BPC* p : bodyPairContacts.v)
        for (Contact* c : p->contactList)
            if (c->fresh) { ordered.push_back(p); p->checked = true; break; }
    // (no picked bodies: interaction is out of scope)
    if (!ordered.empty()) {
        std::vector<BPC*> first = ordered;
        getNextLayer(first, ordered);
    }
    for (BPC* p : bodyPairContacts.v)
        if (!p->checked) { ordered.push_back(p); p->checked = true; }
    for (Body* b : bodies)
        if (b->isCollection && !b->sleeping)
            for (BPC* p : b->bpcs.v)
                if (!p->checked) { ordered.push_back(p); p->checked = true; }
    for (BPC* p : ordered)
        for (Contact* c : p->contactList) out.push_back(c);
}

void World::updateInCollections(double dt) {
    if (!P.update_contacts_in_collections) return;
    alt.clear();
    bool has = false;
    for (Body* b : bodies) if (b->isCollection) has = true;
    if (!has) return;
    if (P.organize_contacts) {
        getOrganizedContacts(alt);
    } else {
        alt = contacts;   // the internalContacts HashSet order is not reproducible; unsupported
    }
    for (Contact* c : alt)
        if (c->body1->parent || c->body2->parent) recomputeJacobian(c, true);
    double comp = P.enable_compliance ? P.compliance : 0.;
    pgs(alt, dt, true, P.iterations_in_collection, P.feedback_stiffness, comp, false);
    for (Body* b : bodies) {
        if (b->isCollection && !b->sleeping)
            for (Body* s : b->bodies)
                if (!s->pinned) {   // RigidBody.advanceVelocities
                    s->v = vscaleadd(dt * s->minv, s->force, s->v);
                    s->v = vadd(s->v, s->dvv);
                    V3 dw = mxv(s->jinv, s->torque);
                    vscale_ip(dw, dt);
                    s->omega = vadd(s->omega, dw);
                    s->omega = vadd(s->omega, s->dvw);
                }
        b->dvv = V3(); b->dvw = V3();
    }
}

// ---------------------------------------------------------------------------
// Motion metric (MotionMetricProcessor.java:39-73), RigidBody.getSpatialVelocity
// (RigidBody.java:458-462)
static V3 spatialVel(const Body* b, const V3& pW) {
    V3 t = vsub(pW, b->x);
    V3 r = vcross(b->omega, t);
    return vadd(r, b->v);
}
static double metric2(const Body* b1, const Body* b2) {
    double largest = 0;
    for (int i = 0; i < 2; i++) {
        const Body* b = i == 0 ? b1 : b2;
        RT T = b->T();
        for (const V3& pt : b->bbB) {
            V3 pW = rt_point(T, pt);
            V3 v1 = spatialVel(b1, pW), v2 = spatialVel(b2, pW);
            v1 = vsub(v1, v2);
            largest = jmax(vlength(v1), largest);
        }
    }
    return largest;
}
static double metric1(const Body* b) {
    double largest = 0;
    RT T = b->T();
    for (const V3& pt : b->bbB) {
        V3 pW = rt_point(T, pt);
        largest = jmax(vlength(spatialVel(b, pW)), largest);
    }
    return largest;
}

// BodyPairContact.accumulateForMerging (BodyPairContact.java:83-121)
void World::accumulateForMerging() {
    for (BPC* p : bodyPairContacts.v) {
        Body* b1 = p->body1->parent ? p->body1->parent : p->body1;
        Body* b2 = p->body2->parent ? p->body2->parent : p->body2;
        double m;
        if (b1->pinned) m = metric1(b2);
        else if (b2->pinned) m = metric1(b1);
        else m = metric2(b1, b2);
        p->motionMetricHist.push_back(m);
        if ((int)p->motionMetricHist.size() > P.step_accum_merging) p->motionMetricHist.erase(p->motionMetricHist.begin());
        int notOnEdge = 0;
        for (Contact* c : p->contactList) if (c->state != ONEDGE) notOnEdge++;
        int st;
        if (notOnEdge == 0) st = ONEDGE;
        else if (notOnEdge >= 2) st = CLEAR;
        else if (p->contactList.size() == 1) st = CLEAR;
        else st = ONEDGE;
        p->contactStateHist.push_back(st);
        if ((int)p->contactStateHist.size() > P.step_accum_merging) p->contactStateHist.erase(p->contactStateHist.begin());
    }
}

// RigidBodySystem.accumulateForUnmerging + BodyPairContact.accumulateForUnmerging
// (RigidBodySystem.java:325-335, BodyPairContact.java:127-145)
void World::accumulateForUnmerging() {
    for (Body* b : bodies) {
        if (!b->isCollection || b->sleeping) continue;
        for (BPC* p : b->bpcs.v) {
            if (!(p->body1->parent && p->body1->parent == p->body2->parent)) continue;
            double m;
            if (p->body1->pinned) m = metric1(p->body2);
            else if (p->body2->pinned) m = metric1(p->body1);
            else m = metric2(p->body1, p->body2);
            if (m > P.threshold_unmerge) p->motionMetricHist.push_back(m);
            else p->motionMetricHist.clear();
        }
    }
}

// ---------------------------------------------------------------------------
// RigidCollection (RigidCollection.java)
static bool sameColl(const Body* a, const Body* b) { return a->parent && a->parent == b->parent; }

static M3 getOp(const Body* b, const V3& com) {   // RigidCollection.getOp (:809-830)
    double x = b->x.x - com.x, y = b->x.y - com.y, z = b->x.z - com.z;
    double x2 = x * x, y2 = y * y, z2 = z * z;
    M3 op;
    op.m00 = y2 + z2; op.m01 = -x * y; op.m02 = -x * z;
    op.m10 = -y * x; op.m11 = x2 + z2; op.m12 = -y * z;
    op.m20 = -z * x; op.m21 = -z * y; op.m22 = x2 + y2;
    return mscale(op, b->massLinear);
}

void World::collUpdateState(Body* c, Body* b) {    // updateCollectionState (:459-469)
    c->pinned = c->pinned || b->pinned;
    c->sleeping = c->sleeping || b->sleeping;
    b->sleeping = false;
}

void World::collUpdateBB(Body* c, Body* b) {       // updateBB(RigidBody) (:637-668)
    if (c->bbB.empty()) return;
    V3 mx(-1.79769313486231570e308, -1.79769313486231570e308, -1.79769313486231570e308);
    V3 mn(1.79769313486231570e308, 1.79769313486231570e308, 1.79769313486231570e308);
    if (b->type == AM_PLANE && !b->isCollection) return;
    for (int i = 0; i < 2; i++) {
        Body* q = i == 0 ? c : b;
        RT T = q->T();
        for (const V3& pt : q->bbB) {
            V3 p = rt_point(T, pt);
            mn.x = std::min(mn.x, p.x); mn.y = std::min(mn.y, p.y); mn.z = std::min(mn.z, p.z);
            mx.x = std::max(mx.x, p.x); mx.y = std::max(mx.y, p.y); mx.z = std::max(mx.z, p.z);
        }
    }
    c->bbB[4] = mn;
    c->bbB[5] = V3(mn.x, mx.y, mx.z);
    c->bbB[6] = V3(mx.x, mn.y, mx.z);
    c->bbB[7] = V3(mx.x, mx.y, mn.z);
    c->bbB[0] = mx;
    c->bbB[1] = V3(mx.x, mn.y, mn.z);
    c->bbB[2] = V3(mn.x, mx.y, mn.z);
    c->bbB[3] = V3(mn.x, mn.y, mx.z);
}

void World::collUpdateBBAll(Body* c) {             // updateBB() (:601-631)
    if (c->bbB.empty()) return;
    V3 mx(-1.79769313486231570e308, -1.79769313486231570e308, -1.79769313486231570e308);
    V3 mn(1.79769313486231570e308, 1.79769313486231570e308, 1.79769313486231570e308);
    for (Body* b : c->bodies) {
        if (b->type == AM_PLANE) continue;
        for (const V3& pt : b->bbB) {
            V3 p = rt_point(b->B2C, pt);
            mn.x = std::min(mn.x, p.x); mn.y = std::min(mn.y, p.y); mn.z = std::min(mn.z, p.z);
            mx.x = std::max(mx.x, p.x); mx.y = std::max(mx.y, p.y); mx.z = std::max(mx.z, p.z);
        }
    }
    c->bbB[4] = mn;
    c->bbB[5] = V3(mn.x, mx.y, mx.z);
    c->bbB[6] = V3(mx.x, mn.y, mx.z);
    c->bbB[7] = V3(mx.x, mx.y, mn.z);
    c->bbB[0] = mx;
    c->bbB[1] = V3(mx.x, mn.y, mn.z);
    c->bbB[2] = V3(mn.x, mx.y, mn.z);
    c->bbB[3] = V3(mn.x, mn.y, mx.z);
}

void World::collAddInternal(Body* c, Body* b) {    // addBodyInternalMethod (:477-514)
    RT tmpT = c->T();
    c->theta = M3::identity();                      // updateTheta
    if (c->pinned) {
        c->v = V3(); c->omega = V3();
        c->massAngular = M3(); c->massAngular0 = M3(); c->jinv = M3(); c->jinv0 = M3();
        c->massLinear = 0; c->minv = 0;
    } else {
        V3 com = c->x;
        vscale_ip(com, c->massLinear);
        com = vscaleadd(b->massLinear, b->x, com);
        double tmi = 1. / (b->massLinear + c->massLinear);
        vscale_ip(com, tmi);
        // updateVelocitiesFrom
        vscale_ip(c->v, c->massLinear);
        c->v = vscaleadd(b->massLinear, b->v, c->v);
        vscale_ip(c->v, tmi);
        vscale_ip(c->omega, c->massLinear);
        c->omega = vscaleadd(b->massLinear, b->omega, c->omega);
        vscale_ip(c->omega, tmi);
        // updateInertia
        M3 m0;
        for (int i = 0; i < 2; i++) {
            Body* q = i == 0 ? c : b;
            m0 = madd(m0, q->massAngular);
            m0 = madd(m0, getOp(q, com));
        }
        c->massAngular = m0;
        collUpdateBB(c, b);
        c->massLinear += b->massLinear;
        c->minv = tmi;
        c->x = com;
        RT T = c->T();
        for (V3& pt : c->bbB) pt = rt_inv_point(T, pt);
    }
    c->B2C = rt_multAinvB(c->T(), tmpT);
}

void World::collInertiaRestInvert(Body* c) {       // updateInertiaRestAndInvert (:674-680)
    if (!c->pinned) {
        minvert(c->massAngular, c->jinv);
        c->massAngular0 = rtmr(c->theta, c->massAngular);
        c->jinv0 = rtmr(c->theta, c->jinv);
    }
}

static void updateRotInertia(Body* b) {           // RigidBody.updateRotationalInertiaFromTransformation (:311-321)
    if (!b->pinned) {
        b->massAngular = rm0rt(b->theta, b->massAngular0);
        b->jinv = rm0rt(b->theta, b->jinv0);
    }
}

void World::collBodiesTransforms(Body* c) {        // updateBodiesTransformations (:588-591)
    for (Body* b : c->bodies) b->B2C = rt_multAinvB(c->T(), b->T());
}

void World::collAddBody(Body* c, Body* b) {        // addBody (:128-139)
    b->parent = c;
    c->bodies.push_back(b);
    collUpdateState(c, b);
    collAddInternal(c, b);
    collInertiaRestInvert(c);
    updateRotInertia(c);
    collBodiesTransforms(c);
}

void World::collAddBodies(Body* c, const std::vector<Body*>& bs) {  // addBodies (:145-158)
    for (Body* b : bs) {
        b->parent = c;
        c->bodies.push_back(b);
        collUpdateState(c, b);
        collAddInternal(c, b);
    }
    collInertiaRestInvert(c);
    updateRotInertia(c);
    collBodiesTransforms(c);
}

void World::collAddCollection(Body* c, Body* o) {  // addCollection (:164-178)
    for (Body* b : o->bodies) { b->parent = c; c->bodies.push_back(b); }
    collUpdateState(c, o);
    collAddInternal(c, o);
    collInertiaRestInvert(c);
    updateRotInertia(c);
    collBodiesTransforms(c);
}

Body* World::newCollection(Body* b1, Body* b2) {   // RigidCollection(body1, body2) (:55-76)
    store.emplace_back();
    Body* c = &store.back();
    c->id = (int)store.size() - 1;
    c->isCollection = true;
    c->type = -1;
    c->theta = M3::identity();
    auto setFrom = [&](Body* b) {                   // RigidBody.set (RigidBody.java:248-271)
        c->v = b->v; c->omega = b->omega; c->x = b->x; c->theta = b->theta;
        c->massLinear = b->massLinear; c->minv = b->minv;
        c->massAngular = b->massAngular; c->massAngular0 = b->massAngular0;
        c->jinv = b->jinv; c->jinv0 = b->jinv0;
        c->pinned = b->pinned; c->sleeping = b->sleeping;
        c->bbB = b->bbB;
    };
    if (b1->type == AM_PLANE && !b1->isCollection) {
        setFrom(b2);
        b2->parent = c;
        c->bodies.push_back(b2);
        collAddBody(c, b1);
    } else {
        setFrom(b1);
        b1->parent = c;
        c->bodies.push_back(b1);
        collAddBody(c, b2);
    }
    return c;
}

void World::collRemoveBodies(Body* c, const std::vector<Body*>& rm) {  // removeBodies (:686-753)
    std::vector<Body*> keep;
    for (Body* b : c->bodies)
        if (std::find(rm.begin(), rm.end(), b) == rm.end()) keep.push_back(b);
    c->bodies = keep;
    RT tmpT = c->T();
    bool wasPinned = c->pinned;
    c->pinned = false;
    for (Body* b : c->bodies) c->pinned = c->pinned || b->pinned;
    c->theta = M3::identity();
    if (c->pinned) {
        c->v = V3(); c->omega = V3();
        c->massAngular = M3(); c->massAngular0 = M3(); c->jinv = M3(); c->jinv0 = M3();
        c->massLinear = 0; c->minv = 0;
    } else if (wasPinned) {
        c->x = V3();
        c->massLinear = 0;
        for (Body* b : c->bodies) { c->x = vscaleadd(b->massLinear, b->x, c->x); c->massLinear += b->massLinear; }
        c->minv = 1. / c->massLinear;
        vscale_ip(c->x, c->minv);
        c->massAngular = M3();                      // computeInertia (:764-772)
        for (Body* b : c->bodies) { c->massAngular = madd(c->massAngular, b->massAngular); c->massAngular = madd(c->massAngular, getOp(b, c->x)); }
        collInertiaRestInvert(c);
    } else {
        for (Body* b : rm) {
            V3 com = c->x;
            vscale_ip(com, c->massLinear);
            c->x = vscaleadd(-b->massLinear, b->x, com);
            vscale_ip(com, 1. / c->massLinear);
            c->massLinear -= b->massLinear;
            c->minv = 1. / c->massLinear;
            vscale_ip(c->x, c->minv);
            // updateInertiaReverse (:797-806)
            c->massAngular = msub(c->massAngular, b->massAngular);
            for (int i = 0; i < 2; i++) {
                Body* q = i == 0 ? c : b;
                c->massAngular = msub(c->massAngular, getOp(q, com));
            }
        }
        collInertiaRestInvert(c);
    }
    updateRotInertia(c);
    collBodiesTransforms(c);
    collUpdateBBAll(c);
    c->B2C = rt_multAinvB(c->T(), tmpT);
}

void World::collToInternalContact(Body* c, BPC* bpc) {   // addToInternalContact (:836-847)
    (void)c;
    std::vector<Contact*> copies;
    for (Contact* k : bpc->contactList) {
        persistent.emplace_back();
        Contact* n = &persistent.back();
        n->body1 = k->body1; n->body2 = k->body2; n->bv1 = k->bv1; n->bv2 = k->bv2; n->info = k->info;
        n->cB1 = k->cB1; n->nB1 = k->nB1; n->t1B1 = k->t1B1; n->t2B1 = k->t2B1;
        n->l0 = k->l0; n->l1 = k->l1; n->l2 = k->l2;
        n->jna_v = k->jna_v; n->jna_w = k->jna_w; n->jnb_v = k->jnb_v; n->jnb_w = k->jnb_w;
        n->jt1a_v = k->jt1a_v; n->jt1a_w = k->jt1a_w; n->jt1b_v = k->jt1b_v; n->jt1b_w = k->jt1b_w;
        n->jt2a_v = k->jt2a_v; n->jt2a_w = k->jt2a_w; n->jt2b_v = k->jt2b_v; n->jt2b_w = k->jt2b_w;
        n->state = k->state;
        n->cv = k->cv; n->prevCv = k->prevCv;
        n->fresh = false;
        copies.push_back(n);
    }
    bpc->contactList = copies;
}

void World::collAddBPCs(Body* c, BPC* bpc) {       // addBPCsToCollection (:854-863)
    (void)c;
    addToBodyListsParent(bpc);
    for (int i = 0; i < 2; i++) {
        Body* b = bpc->getBody(i);
        for (BPC* e : b->bpcs.v) addToBodyListsParent(e);
    }
}

void World::collFillInternal(Body* c) {            // fillInternalBodyContacts (:959-978)
    c->bpcs.clear();
    for (Body* b : c->bodies)
        for (BPC* p : b->bpcs.v)
            if (!c->bpcs.contains(p)) {
                c->bpcs.add(p);
                Body* o = p->getOtherBody(b);
                if (sameColl(b, o)) p->inCollection = true;
            }
}

void World::collAddIncomplete(Body* body, std::vector<BPC*>& removal) {  // addIncompleteContacts (:987-998)
    std::vector<BPC*> snap = body->bpcs.v;
    for (BPC* p : snap) {
        if (sameColl(p->body1, p->body2) && !p->inCollection) {
            p->inCollection = true;
            p->motionMetricHist.clear();
            p->contactStateHist.clear();
            collToInternalContact(body->parent, p);
            collAddBPCs(body->parent, p);
            removal.push_back(p);
        }
    }
}

void World::collApplyVelocitiesTo(Body* c, Body* b) {   // applyVelocitiesTo (:925-937)
    V3 r = vsub(b->x, c->x);
    V3 wxr = vcross(c->omega, r);
    b->v = vadd(c->v, wxr);
    b->omega = c->omega;
}

void World::collUnmergeBody(Body* c, Body* b) {    // unmergeBody (:944-953)
    collApplyVelocitiesTo(c, b);
    b->dvv = V3(); b->dvw = V3();
    b->parent = nullptr;
}

void World::collUpdateBodiesPositions(Body* c) {   // updateBodiesPositionAndTransformations (:898-909)
    for (Body* b : c->bodies) {
        RT T = rt_mult(c->T(), b->B2C);
        b->x = T.t; b->theta = T.R;
        if (!c->pinned) {
            b->jinv = rm0rt(b->theta, b->jinv0);
            b->massAngular = rm0rt(b->theta, b->massAngular0);
        }
    }
}

// ---------------------------------------------------------------------------
// Merging (Merging.java:73-163, 215-393)
// A body with a prescribed motion never merges: a collection that holds a
// pinned body stays put, so the body's motion would stop acting on its
// contacts while it moved through the members merged with it.  The
// reference's pinned bodies never move, and this test is the only addition.
static bool kinematicPair(const std::vector<World::Kinematic>& kin, const BPC* p) {
    for (const World::Kinematic& q : kin)
        if (q.body == p->body1 || q.body == p->body2) return true;
    return false;
}

static bool checkMergeCondition(const am_params& P, const std::vector<World::Kinematic>& kin,
                                BPC* p) {   // BodyPairContact.java:151-177
    if (kinematicPair(kin, p)) return false;
    if (p->body1->sleeping && p->body2->sleeping) return true;
    if (P.enable_merge_let_it_breathe)
        for (Contact* c : p->contactList)
            if (std::fabs(c->prevCv - c->cv) > P.threshold_breath) return false;
    if (!P.enable_merge_pinned && (p->body1->pinned || p->body2->pinned)) return false;
    if (sameColl(p->body1, p->body2)) return false;
    if ((int)p->motionMetricHist.size() == P.step_accum_merging) {
        for (double m : p->motionMetricHist) if (m > P.threshold_merge) return false;
    } else return false;
    if (P.enable_merge_stable_contact) {
        if ((int)p->contactStateHist.size() == P.step_accum_merging) {
            for (int s : p->contactStateHist) if (s == ONEDGE) return false;
        } else return false;
    }
    return true;
}

bool World::mergeTest(BPC* p) const { return checkMergeCondition(P, kin, p); }

bool World::unmergeTest(BPC* p) const {   // the selection in Merging.unmerge (:222-240)
    for (Contact* c : p->contactList) {
        if (c->state == BROKEN && P.enable_unmerge_normal) return true;
        if (c->state == ONEDGE && P.enable_unmerge_friction) return true;
    }
    return (int)p->motionMetricHist.size() >= P.step_accum_unmerging && p->contactList.size() < 3;
}

static void listRemove(std::vector<Body*>& v, Body* b) {
    for (size_t i = 0; i < v.size(); i++) if (v[i] == b) { v.erase(v.begin() + i); return; }
}

void World::merge() {
    if (!P.enable_merging) return;
    std::vector<BPC*> removal;
    for (BPC* p : bodyPairContacts.v) {
        if (p->inCollection || !checkMergeCondition(P, kin, p)) continue;
        mergingEvent = true;
        mergeEvents++;
        p->inCollection = true;
        p->motionMetricHist.clear();
        p->contactStateHist.clear();
        removal.push_back(p);
        Body* b1 = p->body1;
        Body* b2 = p->body2;
        if (!b1->parent && !b2->parent) {
            listRemove(bodies, b1);
            listRemove(bodies, b2);
            Body* c = newCollection(b1, b2);
            collToInternalContact(c, p);
            collAddBPCs(c, p);
            bodies.push_back(c);
        } else if (b1->parent && b2->parent) {
            Body* big = b1->parent;
            Body* small = b2->parent;
            if (!(b1->parent->bodies.size() > b2->parent->bodies.size())) { big = b2->parent; small = b1->parent; }
            listRemove(bodies, small);
            for (BPC* q : small->bpcs.v) big->bpcs.add(q);
            collAddCollection(big, small);
            collToInternalContact(big, p);
            // body2.parent already points at the merged collection here, so the
            // reference walks every body of the merged collection
            std::vector<Body*> all = big->bodies;
            for (Body* b : all) collAddIncomplete(b, removal);
            collAddBPCs(big, p);
        } else if (b1->parent) {
            listRemove(bodies, b2);
            collAddBody(b1->parent, b2);
            collToInternalContact(b1->parent, p);
            collAddIncomplete(b2, removal);
            collAddBPCs(b1->parent, p);
        } else {
            listRemove(bodies, b1);
            collAddBody(b2->parent, b1);
            collToInternalContact(b2->parent, p);
            collAddIncomplete(b1, removal);
            collAddBPCs(b2->parent, p);
        }
    }
    for (BPC* p : removal) bodyPairContacts.remove(p);
}

void World::buildNeighbor(Body* b, OSet<Body*>& sub, OSet<Body*>& handled) {  // buildNeighborBody (:381-393)
    for (BPC* p : b->bpcs.v) {
        if (!p->inCollection) continue;
        Body* o = p->getOtherBody(b);
        if (!sub.contains(o) && !handled.contains(o)) {
            sub.add(o);
            buildNeighbor(o, sub, handled);
        }
    }
}

bool World::unmergeSelected(Body* coll, OSet<BPC*>& sel, std::vector<Body*>& newBodies) {  // unmergeSelectedBpcs (:286-374)
    bool removeCollection = true;
    for (BPC* p : sel.v) p->inCollection = false;
    OSet<Body*> handled, sub, remained;
    std::vector<Body*> snapshot = coll->bodies;
    for (Body* b : snapshot) {
        if (handled.contains(b)) continue;
        sub.add(b);
        buildNeighbor(b, sub, handled);
        for (Body* q : sub.v) handled.add(q);
        if (coll->bodies.size() != sub.size()) {
            if (sub.size() < coll->bodies.size() / 2 + 1) {
                for (Body* q : sub.v) collUnmergeBody(coll, q);
                if (sub.size() > 1) {
                    Body* sb1 = sub.v[0];
                    Body* sb2 = sub.v[1];
                    std::vector<Body*> rest(sub.v.begin() + 2, sub.v.end());
                    Body* nc = newCollection(sb1, sb2);
                    collAddBodies(nc, rest);
                    collFillInternal(nc);
                    newBodies.push_back(nc);
                } else if (sub.size() == 1) {
                    newBodies.push_back(sub.v[0]);
                }
            } else {
                removeCollection = false;
                for (Body* q : sub.v) remained.add(q);
            }
        } else {
            removeCollection = false;
            for (Body* q : sub.v) remained.add(q);
            break;
        }
        sub.clear();
    }
    for (BPC* p : sel.v) {
        if (sameColl(p->body1, p->body2)) {
            p->inCollection = true;
        } else {
            if (!bodyPairContacts.contains(p)) {
                bodyPairContacts.add(p);
                for (Contact* c : p->contactList) {
                    c->l0w = c->l0; c->l1w = c->l1; c->l2w = c->l2;
                    contacts.push_back(c);
                }
            }
            p->motionMetricHist.clear();
            p->contactStateHist.clear();
        }
    }
    if (!removeCollection) {
        if (remained.size() != coll->bodies.size()) {
            std::vector<Body*> rm;
            for (Body* q : handled.v) if (!remained.contains(q)) rm.push_back(q);
            collRemoveBodies(coll, rm);
            collFillInternal(coll);
        }
    }
    return removeCollection;
}

void World::unmerge() {   // Merging.unmerge (:215-273)
    if (!P.enable_unmerging) return;
    if (!P.enable_unmerge_relative_motion && !P.enable_unmerge_normal && !P.enable_unmerge_friction) return;
    std::vector<Body*> removalQ, additionQ;
    std::vector<Body*> snapshot = bodies;
    for (Body* b : snapshot) {
        if (b->sleeping) continue;
        if (!b->isCollection) continue;
        OSet<BPC*> sel;
        for (BPC* p : b->bpcs.v) {
            if (!p->inCollection) continue;
            if (sel.contains(p)) continue;
            bool state = false;   // checkContactsState (BodyPairContact.java:255-266)
            for (Contact* c : p->contactList) {
                if (c->state == BROKEN && P.enable_unmerge_normal) { state = true; break; }
                if (c->state == ONEDGE && P.enable_unmerge_friction) { state = true; break; }
            }
            bool motion = (int)p->motionMetricHist.size() >= P.step_accum_unmerging && p->contactList.size() < 3;
            if (!state && !motion) continue;
            sel.add(p);    // addBpcToUnmerge
        }
        std::vector<Body*> nb;
        bool removeC = false;
        if (!sel.empty()) removeC = unmergeSelected(b, sel, nb);
        if (!nb.empty()) {
            mergingEvent = true;
            unmergeEvents++;
            for (Body* q : nb) additionQ.push_back(q);
            if (removeC) removalQ.push_back(b);
        }
    }
    for (Body* q : additionQ) bodies.push_back(q);
    if (!removalQ.empty()) {
        std::vector<Body*> keep;
        for (Body* q : bodies)
            if (std::find(removalQ.begin(), removalQ.end(), q) == removalQ.end()) keep.push_back(q);
        bodies = keep;
    }
}

// ---------------------------------------------------------------------------
// Sleeping (Sleeping.java:49-160)
static void wakeBody(Body* b) {   // RigidBody.wake (RigidBody.java:298-306)
    if (b->sleeping) { b->sleeping = false; b->metricHistory.clear(); }
    if (b->parent) wakeBody(b->parent);
}

void World::wake() {
    if (!P.enable_sleeping) return;
    for (Body* b : bodies) {
        if (!b->sleeping) continue;
        std::vector<BPC*> snap = b->bpcs.v;
        for (BPC* p : snap)
            if (!p->inCollection && !(p->body1->pinned || p->body2->pinned)) { wakeBody(p->body1); wakeBody(p->body2); }
    }
}

void World::sleep() {
    if (!P.enable_sleeping) return;
    double thr = P.sleep_threshold;
    for (Body* b : bodies) {
        if (b->sleeping) continue;
        bool external = false;
        for (BPC* p : b->bpcs.v)
            if (!p->inCollection && !(p->body1->pinned || p->body2->pinned)) { external = true; break; }
        if (external) continue;
        b->metricHistory.push_back(metric1(b));
        if ((int)b->metricHistory.size() > P.sleep_step_accum) b->metricHistory.erase(b->metricHistory.begin());
        bool s = true;
        double prev = 1.79769313486231570e308;
        double eps = 5e-5;
        if ((int)b->metricHistory.size() < P.sleep_step_accum) s = false;
        else
            for (double m : b->metricHistory) {
                if (m > prev + eps) { s = false; break; }
                if (m > thr) { s = false; break; }
                prev = m;
            }
        b->sleeping = s;
    }
}

// ---------------------------------------------------------------------------
// RigidBodySystem (RigidBodySystem.java:102-185, 190-202, 276-290, 342-352, 428-436)
void World::clearBodies() {
    for (Body* b : bodies) {
        b->force = V3(); b->torque = V3(); b->dvv = V3(); b->dvw = V3();
        if (b->isCollection)
            for (Body* s : b->bodies) {   // RigidCollection.clearBodies
                collApplyVelocitiesTo(b, s);
                s->force = V3(); s->torque = V3(); s->dvv = V3(); s->dvw = V3();
            }
    }
}

void World::applyExternalForces() {
    if (!P.use_gravity) return;
    double th = P.gravity_angle / 180.0 * M_PI;
    double g = P.gravity_amount;
    V3 dir(g * std::cos(th), g * std::sin(th), 0);
    for (Body* b : bodies) {
        b->force = vadd(b->force, vscale(-b->massLinear, dir));
        if (b->isCollection)
            for (Body* s : b->bodies) s->force = vadd(s->force, vscale(-s->massLinear, dir));
    }
}

static void advanceVel(Body* b, double dt) {   // RigidBody.advanceVelocities (:409-417)
    b->v = vscaleadd(dt * b->minv, b->force, b->v);
    b->v = vadd(b->v, b->dvv);
    V3 dw = mxv(b->jinv, b->torque);
    vscale_ip(dw, dt);
    b->omega = vadd(b->omega, dw);
    b->omega = vadd(b->omega, b->dvw);
}

static void advancePos(Body* b, double dt) {   // RigidBody.advancePositions (:427-441)
    b->x = vscaleadd(dt, b->v, b->x);
    double t = vlength(b->omega) * dt;
    V3 w = b->omega;
    vnormalize(w);
    if (t > 1e-8) {
        double s, c;
        det_sincos(t, &s, &c);
        double c1 = 1 - c;
        M3 R;   // expRodrigues (:382-401)
        R.m00 = c + w.x * w.x * c1;
        R.m10 = w.z * s + w.x * w.y * c1;
        R.m20 = -w.y * s + w.x * w.z * c1;
        R.m01 = -w.z * s + w.x * w.y * c1;
        R.m11 = c + w.y * w.y * c1;
        R.m21 = w.x * s + w.y * w.z * c1;
        R.m02 = w.y * s + w.x * w.z * c1;
        R.m12 = -w.x * s + w.y * w.z * c1;
        R.m22 = c + w.z * w.z * c1;
        b->theta = mnormalizeCP(mmul(R, b->theta));
    }
    updateRotInertia(b);
    if (!b->pinned && b->bbB.size() == 8) {   // updateBBW (:323-328)
        RT T = b->T();
        b->bbMinW = rt_point(T, b->bbB[0]);
        b->bbMaxW = rt_point(T, b->bbB[4]);
    }
}

void World::advanceVelocities(double dt) {
    for (Body* b : bodies)
        if (!b->pinned && !b->sleeping) {
            advanceVel(b, dt);
            if (b->isCollection)   // RigidCollection.advanceVelocities -> applyVelocitiesToBodies
                for (Body* s : b->bodies) collApplyVelocitiesTo(b, s);
        }
}

void World::advancePositions(double dt) {
    for (Body* b : bodies)
        if (!b->pinned && !b->sleeping) {
            advancePos(b, dt);
            if (b->isCollection) collUpdateBodiesPositions(b);
        }
}

void World::viscousDecay() {
    for (Body* b : bodies) { vscale_ip(b->v, P.viscous_linear); vscale_ip(b->omega, P.viscous_angular); }
}

// the library's prescribed oscillation of pinned bodies, evaluated with the
// same operations: x = x0 + axis * (amp * sin(w n dt)), v = axis * ((amp * w)
// * cos(w n dt)) at the start of the n-th step
void World::applyKinematic() {
    if (kin.empty()) return;
    for (const Kinematic& q : kin) {
        const double t = (double)kinSteps * q.dt;
        double sn, cs;
        det_sincos(q.omega * t, &sn, &cs);
        double x[3], v[3];
        for (int k = 0; k < 3; k++) {
            x[k] = q.x0[k] + q.axis[k] * (q.amp * sn);
            v[k] = q.axis[k] * ((q.amp * q.omega) * cs);
        }
        q.body->x = V3(x[0], x[1], x[2]);
        q.body->v = V3(v[0], v[1], v[2]);
    }
    kinSteps++;
}

void World::step(double dt) {
    applyKinematic();
    totalSteps++;
    clearBodies();
    applyExternalForces();
    updateContactsMap();
    collisionDetection();
    updateBodyPairContacts();
    warmStart();
    wake();
    updateInCollections(dt);
    accumulateForUnmerging();
    unmerge();
    if (mergingEvent) {
        for (Body* b : bodies) { b->force = V3(); b->torque = V3(); b->dvv = V3(); b->dvw = V3(); }
        applyExternalForces();
    }
    if (P.warm_start) redoWarmStart();
    else for (Contact* c : contacts) { c->l0 = c->l1 = c->l2 = 0; }
    solveLCP(dt);
    clearBodyPairContacts();
    advanceVelocities(dt);
    accumulateForMerging();
    advancePositions(dt);
    if ((totalSteps % P.steps_between_merge_events) == 0) merge();
    sleep();
    viscousDecay();
}

}  // namespace orc
