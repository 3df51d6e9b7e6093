// oracle.hpp -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the reference's
// per-step contact path (EulalieCoevoet/AdaptiveMerging, src/mergingBodies3D),
// used by tests/ to check the device path and by bench.py as the CPU baseline.
// Nothing in the product links or calls this code.
//
// Parity unpinned: the reference is Java with no tests or golden vectors for
// the 3D engine, and it cannot run here (no JDK, missing JOGL jar), so the
// restatement follows the Java sources line by line (cited per function in
// oracle.cpp) with javax.vecmath operation order (vm.hpp), and is held by
// analytic known answers, invariants and its own committed fixture
// (tests/test_oracle_cpu.py, tests/golden/).  Identity-hashed
// Java HashSets are replaced by insertion-ordered sets (LinkedHashSet order),
// which is the documented deterministic order of every parity test.
#pragma once
#include <cstdint>
#include <deque>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../include/am.h"
#include "vm.hpp"

namespace orc {

struct Body;
struct BPC;

// A composite body (RigidBodyGeomComposite, XMLParser.createComposite): a
// rigid body whose geometry is a list of box and sphere sub-bodies
// (am_scene's sub-body arrays).
constexpr int ORC_COMPOSITE = AM_COMPOSITE;
// ids of composite sub-bodies (the csb1 / csb2 of Contact), apart from the
// scene bodies and collections
constexpr int ORC_SUB_ID0 = 1 << 24;

// Insertion-ordered set (LinkedHashSet semantics: remove + add moves to end).
template <class T>
struct OSet {
    std::vector<T> v;
    std::unordered_set<T> s;
    bool contains(T x) const { return s.count(x) != 0; }
    bool add(T x) {
        if (s.count(x)) return false;
        s.insert(x); v.push_back(x); return true;
    }
    bool remove(T x) {
        if (!s.count(x)) return false;
        s.erase(x);
        for (size_t i = 0; i < v.size(); i++) if (v[i] == x) { v.erase(v.begin() + i); break; }
        return true;
    }
    void clear() { v.clear(); s.clear(); }
    size_t size() const { return v.size(); }
    bool empty() const { return v.empty(); }
};

struct Node {            // BVNode + BVSphere
    V3 cB, cW;
    double r = 0;
    Body* body = nullptr;
    int child0 = -1, nchild = 0;
    int id = 0;
};

enum ContactState { BROKEN = 0, ONEDGE = 1, CLEAR = 2 };

struct Contact {         // Contact.java
    Body* body1 = nullptr;
    Body* body2 = nullptr;
    int bv1 = AM_BV_NULL, bv2 = AM_BV_NULL;
    int info = 0;
    V3 cB1, nB1, t1B1, t2B1;
    double cv = 0, prevCv = 0;
    int state = CLEAR;
    bool fresh = false;
    V3 jna_v, jna_w, jnb_v, jnb_w, jt1a_v, jt1a_w, jt1b_v, jt1b_w, jt2a_v, jt2a_w, jt2b_v, jt2b_w;
    double l0 = 0, l1 = 0, l2 = 0, l0w = 0, l1w = 0, l2w = 0;
    double bn = 0, bt1 = 0, bt2 = 0, D00 = 0, D11 = 0, D22 = 0, w1 = 0, w2 = 0;
    int csb1 = -1, csb2 = -1;    // ids of the composite sub-bodies that touched (csb1 / csb2), -1: none
};

struct Body {            // RigidBody.java / PlaneRigidBody.java / RigidCollection.java
    int id = 0;
    int type = AM_BOX;
    bool isCollection = false;
    bool pinned = false, sleeping = false;
    bool magnetic = false, activateMagnet = false;
    double massLinear = 0, minv = 0;
    M3 massAngular0, massAngular, jinv0, jinv;
    V3 force, torque, x, v, omega;
    M3 theta;
    V3 dvv, dvw;                       // deltaV
    std::vector<V3> bbB;               // boundingBoxB
    V3 bbMinW, bbMaxW;
    double friction = 0.8, restitution = 0, radius = 0;
    V3 size;                           // box
    V3 pn, pp; double pd = 0;          // plane
    int root = -1;
    Body* parent = nullptr;
    RT B2C;                            // transformB2C
    OSet<BPC*> bpcs;                   // bodyPairContacts
    std::vector<double> metricHistory;
    std::vector<Body*> bodies;         // RigidCollection.bodies
    std::vector<Body*> subs;           // RigidBodyGeomComposite.bodies
    Body* compParent = nullptr;        // compositeBodyParent of a sub-body
    RT B2Cc;                           // a sub-body's transformB2C (pose in its composite)
    RT T() const { return RT{theta, x}; }
};

struct BPC {             // BodyPairContact.java
    Body* body1;
    Body* body2;
    std::vector<Contact*> contactList;
    std::vector<double> motionMetricHist;
    std::vector<int> contactStateHist;
    bool inCollection = false;
    bool checked = false;
    Body* getBody(int i) const { return i == 0 ? body1 : body2; }
    Body* getOtherBody(Body* b) const { return body1 == b ? body2 : (body2 == b ? body1 : nullptr); }
};

// Contact.hashCode/equals (Contact.java:543-572): unordered (body, bv,
// composite sub-body) pair plus info.
struct CKey {
    int a, bva, b, bvb, info, csba = -1, csbb = -1;
    bool operator==(const CKey& o) const {
        return a == o.a && bva == o.bva && b == o.b && bvb == o.bvb && info == o.info && csba == o.csba &&
               csbb == o.csbb;
    }
};
struct CKeyHash {
    size_t operator()(const CKey& k) const {
        uint64_t h = (uint64_t)(uint32_t)k.a * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(uint32_t)k.bva + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k.b * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k.bvb + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k.info * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k.csba + ((uint64_t)(uint32_t)k.csbb << 32) + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
inline CKey ckey(const Contact* c, int info) {
    CKey k;
    int a = c->body1->id, b = c->body2->id;
    if (a < b || (a == b && (c->bv1 < c->bv2 || (c->bv1 == c->bv2 && c->csb1 <= c->csb2)))) {
        k.a = a; k.bva = c->bv1; k.b = b; k.bvb = c->bv2; k.csba = c->csb1; k.csbb = c->csb2;
    } else {
        k.a = b; k.bva = c->bv2; k.b = a; k.bvb = c->bv1; k.csba = c->csb2; k.csbb = c->csb1;
    }
    k.info = info;
    return k;
}

struct Stats {
    int sweeps = 0;
    double last_change = 0;
};

struct World {
    am_params P;
    // Stop of the full solve at a relative natural-map residual (not part of
    // the reference, which stops on max |delta lambda| only): checked every
    // resCheck sweeps when resTarget > 0.
    double resTarget = 0;
    int resCheck = 0;
    std::deque<Body> store;            // stable storage; scene bodies first
    std::vector<Body*> bodies;         // RigidBodySystem.bodies (top level)
    std::vector<Node> nodes;
    int nScene = 0;
    std::deque<BPC> bpcStore;
    OSet<BPC*> bodyPairContacts;       // CollisionProcessor.bodyPairContacts
    // contacts: two pools + persistent copies for collections
    std::deque<Contact> pool[2];
    int cur = 0;
    std::deque<Contact> persistent;
    std::vector<Contact*> contacts;    // CollisionProcessor.contacts
    std::vector<Contact*> alt;         // altContactList
    std::unordered_map<CKey, Contact*, CKeyHash> last;  // lastTimeStepContacts
    std::unordered_map<uint64_t, BPC*> bpcIndex;   // speeds checkExists (same result as the linear search)
    bool mergingEvent = false;
    int totalSteps = 0;
    // pinned bodies with a prescribed oscillation (the library's
    // am_set_kinematic; not part of the reference)
    struct Kinematic { Body* body; double x0[3], axis[3], amp, omega, dt; };
    std::vector<Kinematic> kin;
    int kinSteps = 0;
    void applyKinematic();
    Stats stats;
    int64_t mergeEvents = 0, unmergeEvents = 0;
    double gdir[3];

    void init(const am_params& p, const am_scene& s);
    // composite bodies: sub-bodies in their own store, placed from their
    // parents before every collision pass (updateBodyPositionsFromParent)
    std::deque<Body> subStore;
    int badSubs = 0;   // sub-bodies refused at init (bad parent or type)
    int addCompositeSub(int parent, int type, const double* shape, const double* R, const double* t);
    void updateCompositeSubs();
    // steps (RigidBodySystem.advanceTime and its phases)
    void step(double dt);
    void clearBodies();
    void applyExternalForces();
    void updateContactsMap();
    void collisionDetection();
    void updateBodyPairContacts();
    void warmStart();
    void wake();
    void updateInCollections(double dt);
    void accumulateForUnmerging();
    void unmerge();
    void redoWarmStart();
    void solveLCP(double dt);
    void clearBodyPairContacts();
    void advanceVelocities(double dt);
    void accumulateForMerging();
    void advancePositions(double dt);
    void merge();
    void sleep();
    void viscousDecay();
    // helpers
    Contact* newContact();
    void narrowPhase(Body* b1, Body* b2);
    void emit(Body* b1, Body* b2, const V3& pW, const V3& nW, int bv1, int bv2, int info, double cv);
    void boxBox(Body* b1, Body* b2);
    void boxPlane(Body* box, Body* plane);
    void boxSphere(Body* box, Body* sph, const V3& c, double r);
    bool boxSphereTest(Body* box, const V3& c, double r);
    void treePlane(int node, Body* b, Body* plane);
    void boxTree(int node, Body* box, Body* tree);
    void treeTree(int n1, int n2, Body* b1, Body* b2);
    void pgs(std::vector<Contact*>& list, double dt, bool inColl, int iters, double fb, double comp, bool early);
    double relResidual(std::vector<Contact*>& list, double comp);
    void updateBPCsForContact(Contact* c);
    void removeEmptyBodyPairContacts();
    void getOrganizedContacts(std::vector<Contact*>& out);
    void getNextLayer(std::vector<BPC*>& layer, std::vector<BPC*>& ordered);
    bool unmergeSelected(Body* coll, OSet<BPC*>& sel, std::vector<Body*>& newBodies);
    void buildNeighbor(Body* b, OSet<Body*>& sub, OSet<Body*>& handled);
    Body* newCollection(Body* b1, Body* b2);
    // collection operations (RigidCollection.java)
    void collAddBody(Body* c, Body* b);
    void collAddBodies(Body* c, const std::vector<Body*>& bs);
    void collAddCollection(Body* c, Body* other);
    void collAddInternal(Body* c, Body* b);
    void collUpdateState(Body* c, Body* b);
    void collUpdateBB(Body* c, Body* b);
    void collUpdateBBAll(Body* c);
    void collInertiaRestInvert(Body* c);
    void collBodiesTransforms(Body* c);
    void collRemoveBodies(Body* c, const std::vector<Body*>& rm);
    void collToInternalContact(Body* c, BPC* bpc);
    void collAddBPCs(Body* c, BPC* bpc);
    void collFillInternal(Body* c);
    void collAddIncomplete(Body* body, std::vector<BPC*>& removal);
    void collUnmergeBody(Body* c, Body* b);
    void collApplyVelocitiesTo(Body* c, Body* b);
    void collUpdateBodiesPositions(Body* c);
    // merge / unmerge predicates of one body-pair contact on the current state
    bool mergeTest(BPC* p) const;
    bool unmergeTest(BPC* p) const;
};

}  // namespace orc
