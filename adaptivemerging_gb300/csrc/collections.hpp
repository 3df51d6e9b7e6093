// collections.hpp -- host-side world mirror and the step context.
//
// HostWorld keeps the per-body records that the host needs to own: the
// top-level body list (RigidBodySystem.bodies), collection membership and the
// derived mass properties computed at load time (XMLParser.java:360-447,
// RigidBody.java:182-206, PlaneRigidBody.java:49-57).  Contacts, pairs and
// the per-step state live on the device.
#pragma once
#include <chrono>
#include <cmath>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"

namespace am {

inline double __longlong_as_double_host(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// am_scene.bbox holds body i's boundingBoxB (six finite numbers)
inline bool given_bbox(const am_scene& s, int i) {
    if (!s.bbox) return false;
    for (int k = 0; k < 6; k++)
        if (!std::isfinite(s.bbox[6 * i + k])) return false;
    return true;
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
    std::vector<int> nbb;                 // bounding-box corners stored (0 for planes)

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
        nbb.assign(cap, 8);
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
                nbb[i] = 0;
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
            } else if (given_bbox(s, i)) {   // sphere tree with its mesh's box
                const double* q = s.bbox + 6 * i;
                ll = mk(q[0], q[1], q[2]); ur = mk(q[3], q[4], q[5]);
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

// insertion-ordered set of ints (LinkedHashSet order: remove + add moves to the end)
struct OSetI {
    std::vector<int> v;
    std::unordered_set<int> s;
    bool contains(int x) const { return s.count(x) != 0; }
    bool add(int x) { if (s.count(x)) return false; s.insert(x); v.push_back(x); return true; }
    bool remove(int x) {
        if (!s.erase(x)) return false;
        for (size_t i = 0; i < v.size(); i++) if (v[i] == x) { v.erase(v.begin() + i); break; }
        return true;
    }
    void clear() { v.clear(); s.clear(); }
    size_t size() const { return v.size(); }
    bool empty() const { return v.empty(); }
};

// host record of a BodyPairContact (BodyPairContact.java:14-45)
struct HBPC {
    int a = -1, b = -1;
    std::vector<int> list;      // contact refs: >= 0 current buffer, < 0 ~slot in the collection store
    std::vector<double> mm;     // motionMetricHist
    std::vector<int> sh;        // contactStateHist
    bool inCollection = false;
    bool checked = false;
};

struct HostMerge {
    std::vector<HBPC> bpc;
    OSetI coll;                                 // CollisionProcessor.bodyPairContacts
    std::vector<OSetI> bodyBpcs;                // RigidBody.bodyPairContacts per body slot
    std::unordered_map<uint64_t, int> index;    // pair -> body-pair contact (checkExists)
    std::vector<int> freeSlots;                 // free slots of the collection contact store
    int nSlots = 0;
    void reset(int cap);
    int findOrCreate(int a, int b);
};

// The step context behind the C ABI.
struct Ctx {
    am_params P;
    int device = -1;             // the CUDA device current when the context was created
    std::string err;
    HostWorld host;
    cudaStream_t stream = nullptr;
    DBodies B;
    DNodes N;
    DContacts C[2];
    int cur = 0;
    DPairs PR;
    int* pairCls = nullptr;      // narrow-phase order: per-class counters
    unsigned* broadMask = nullptr;   // broad phase: hit mask per row and 32-pair chunk
    size_t broadMaskCap = 0;
    // staged narrow phase: raw contacts per pair (7 doubles + 5 ints per slot)
    bool narrowStageable = false;    // no body is a sphere tree of more than one node
    double* stageD = nullptr;
    int* stageI = nullptr;
    size_t stageCap = 0;
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
    std::vector<int> hColOff;    // colour offsets of the coloured full solve (host copy)
    int* hColPin = nullptr;      // pinned staging of the colour offsets (MAXC + 1)
    int nSubIds = 0;             // entries of subIds (members of all collections)
    double* Mj = nullptr;     // coloured sweep: M^-1 J^T per row and lane (36 per contact)
    double* invD = nullptr;   // coloured sweep constants per contact: 1/(D + c), A, q per row, couplings, mu
    int mjCap = 0;
    float* mixF = nullptr;    // AM_ORDER_MIXED: FP32 operands, base constants and corrections (mjCap stride)
    float* mixU = nullptr;    // AM_ORDER_MIXED: FP32 delta-v corrections, 6 per body
    int* mixG = nullptr;      // AM_ORDER_MIXED: group records, 4 ints per coloured group
    int mixFCap = 0, mixUCap = 0, mixGCap = 0;
    int mixedForm = -1, mixedRefine = 0;   // am_set_mixed_form
    double* putStage = nullptr;            // am_put_bodies with collections: staged arrays
    int* putParent = nullptr;              // ... and the collection of every scene body
    size_t putStageCap = 0;
    int mixedLastForm = -1;                // form of the last mixed solve
    int nScene = 0, ntop = 0, nContacts = 0, nPrev = 0, nPairs = 0;
    int totalSteps = 0;
    bool mergingEvent = false;
    am_solve_stats stats{};
    am_perf perf{};
    cudaEvent_t evA = nullptr, evB = nullptr;
    // batched step: device events at the phase boundaries (detection, warm
    // start, solve set-up, sweeps, integration, statistics); per-phase sums
    // since the last am_reset_perf
    cudaEvent_t evPh[7] = {};
    double phaseDevMs[AM_STEP_PHASES] = {};
    bool pgsPending = false;
    std::vector<void*> allocs;
    // merging state
    HostMerge M;
    DContacts I{};      // contacts living inside collections
    DContacts Sw{};     // gathered single-sweep list
    int* idxA = nullptr;
    int* idxB = nullptr;
    int idxCap = 0;
    int* metA = nullptr;
    int* metB = nullptr;
    int* metM = nullptr;
    double* metOut = nullptr;
    int metCap = 0;
    int* nbbDev = nullptr;
    std::vector<double> devDv;
    std::vector<int> keyB1, keyB2, freshH, stateH, istateH;
    std::vector<double> lam0H, cvH, icvH, ipcvH;
    std::vector<int> apA, apB, apOff, apCnt;   // pairs handed back by unmerge this step
    int appended = 0;
    // level-scheduled exact sweep
    int* levOrder = nullptr;
    int* levOff = nullptr;
    int levCap = 0;
    int gsBlocksMax = 0;
    std::vector<int> hS1, hS2, hOrder, hLevOff, hLast;
    // batched scenes (nScenes > 0): concatenated bodies, one CTA per scene in the solve
    int nScenes = 0;
    int maxSceneBodies = 0;
    int* sceneOfDev = nullptr;
    int* sceneBodyOffDev = nullptr;
    int* topEnd = nullptr;
    int* bPairOff = nullptr;
    float* bRec = nullptr;
    int2* bLid = nullptr;        // per group (colour order): scene-local body ids
    int2* bGInfo = nullptr;      // per group (colour order): first slot, contacts
    int* bSlotOf = nullptr;      // contact -> slot (records are stored in colour order)
    int* bContactOf = nullptr;   // slot -> contact
    int* bChunkK = nullptr;      // per scene: chunk heads (group positions), MAXCH + 1 each
    int* bNChunks = nullptr;
    int* bSceneOrder = nullptr;  // CTA -> scene, costliest scenes first (null: identity)
    int* bSceneOrderBuf = nullptr;
    int batchCap = 0;            // records staged per chunk (0: autotune)
    int batchCapUser = 0;        // staging capacity fixed by the caller (0: autotuned)
    int batchResident = 0;       // scenes solved with all records in shared memory, last step
    size_t batchSmemLimit = 0;   // dynamic shared memory the sweep kernel may use
    int batchInner = 1;          // passes over a body pair's contacts per sweep
    int batchClasses = 1;        // small scenes in size-class launches (0: all in the one-CTA launch)
    // per-phase wall times of the last step (the reference's CSV columns), on request
    bool phaseOn = false;
    double phase[AM_NUM_PHASES] = {};
    // wall clock in seconds after the stream's work so far (0 when phase timing is off)
    double phaseNow() {
        if (!phaseOn) return 0.;
        cudaStreamSynchronize(stream);
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }
    void phaseAdd(int k, double t0) { if (phaseOn) phase[k] += phaseNow() - t0; }
    double batchRelax = 1.0;     // over-relaxation of the batched sweep (1: plain projected Gauss-Seidel)
    int batchSym = 0;            // 1: odd sweeps walk the colours backwards
    int batchAccel = 0;          // 1: nonsmooth nonlinear conjugate gradient around each sweep
    double batchCriticalFrac = 0.75;   // scenes within this fraction of the costliest solve are critical
    int batchCriticalCap = 640;        // records per CTA of a critical scene's cluster
    float* bGP = nullptr;        // per slot: g and p of the conjugate-gradient step (streamed scenes)
    float* bDQ = nullptr;        // per body: delta-v at sweep start and q (streamed scenes)
    // scenes larger than one CTA's shared memory: thread-block clusters
    int2* bSceneSize = nullptr;  // per scene: slots, one group per colour (split overhead)
    long long* bTrace = nullptr; // per scene, last solve: start and end (device timer, ns), SM of the (first) CTA
    int* bSceneActive = nullptr; // per scene: bodies in contact (the ones the sweep keeps)
    int* bLidOf = nullptr;       // per body: compact id among its scene's active bodies, -1 if inactive
    int* bBodyOf = nullptr;      // scene body offset + compact id -> body
    std::vector<int> hSmall, hBigK[3];   // one-CTA scenes; clusters of 2, 4, 8 CTAs
    // small resident scenes in size classes: one launch per class, each with
    // shared memory and CTA size for its largest scene, so several CTAs share
    // an SM
    std::vector<int> hClass[10];
    int smallNb = 0, classNb[10] = {};    // largest scene (active bodies) of each launch
    int bigNb[3] = {0, 0, 0}, bigCap[3] = {0, 0, 0};
    size_t clusterSmemLimit = 0;
    std::vector<long long> lastCost;
    int clusterCap = 0;
    int clusterCapUser = 0;      // cluster staging capacity fixed by the caller (0: largest that fits)
    bool clusterEnabled = false, clusterAllowed = true, clusterUsable = false;
    static const int NPOOL = 28;         // sweep launches: one-CTA, 10 size classes, 3 cluster sizes; two parts each
    cudaStream_t pool[NPOOL] = {};
    cudaEvent_t evFork = nullptr, poolJoin[NPOOL] = {};
    float* bLam = nullptr;
    int bRecCap = 0;
    int* bColour = nullptr;
    int* bOrder = nullptr;
    int bPairCap = 0;
    int* bColOff = nullptr;
    int* bSweeps = nullptr;
    float* bRes = nullptr;
    int batchThreads = 0;        // threads per scene CTA in use (0: not tuned yet)
    int batchThreadsUser = 0;    // CTA size fixed by the caller (0: autotuned)
    int batchTunedContacts = 0;  // contacts at the last tuning
    double solveTol = 0.0;       // coloured single-scene solve: relative residual target (0: off)
    int solveCheck = 0;
    double batchTol = 1e-6;      // relative natural-map residual target
    int batchCheck = 10;         // sweeps between residual checks
    long long batchSweepsTotal = 0;
    long long batchContactSweepsLast = 0;
    long long* bCS = nullptr;
    int batchConverged = 0;
    // learned warm start
    float *lW = nullptr, *lG = nullptr, *lM = nullptr, *lV = nullptr, *lNorm = nullptr, *lBias = nullptr,
          *lLoss = nullptr;
    __nv_bfloat16* lWb = nullptr;
    bool lReady = false;         // weights set by am_learned_use / _weights / _train, BF16 copy current
    float *lX = nullptr, *lY = nullptr, *lDX = nullptr, *lDY = nullptr, *lZ1 = nullptr, *lZ2 = nullptr,
          *lYh = nullptr, *lXN = nullptr, *lA1 = nullptr, *lA2 = nullptr, *lD1 = nullptr, *lD2 = nullptr,
          *lDYb = nullptr;
    int *lKeep = nullptr, *lPos = nullptr, *lIdx = nullptr;
    int lFeatCap = 0, lDcap = 0, lDn = 0, lTrainCap = 0, lIdxCap = 0;
    int lCollect = 0, lUse = 0;   // lUse: 0 off, 1 BF16 tensor cores, 2 FP32
    int lScope = 0;               // 0: fresh contacts take the learned start, 1: all contacts
    long long lAdamT = 0;
    int lFallbackScenes = 0;      // scenes re-solved from the plain warm start, last step
    float* bLamL = nullptr;       // learned start, packed like bLam
    int* bFall = nullptr;         // per scene: 1 when it fell back to the plain start
    long long mergeEvents = 0, unmergeEvents = 0;

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
    // pinned bodies moved by a prescribed oscillation (am_set_kinematic)
    static const int MAXKIN = 8;
    struct Kinematic {
        int body;
        double x0[3], axis[3], amp, omega, dt;
    };
    std::vector<Kinematic> kin;
    int kinSteps = 0;   // steps started since the last am_set_kinematic
    void applyKinematic();
    int setKinematic(int body, const double* axis, double amp, double freq, double dt);
    int collisionDetection();
    int warmStart();
    int wake();
    int runPGS(int nc, const int* order, int iters, bool inColl, double dt, bool redoWarm);
    int exactSweep(DContacts& buf, int n, int iters, bool inColl);
    int solveLCP(double dt, bool redoWarm);
    int finishStep(double dt);
    int step(double dt);
    int stepWithMerging(double dt);
    int stepPlain(double dt);
    int collectStats();
    void foldTiming();
    int getBodies(am_body_state* out);
    // merging (merging.cu)
    void addToBodyLists(int p);
    void addToBodyListsParent(int p);
    void removeFromBodyLists(int p);
    void removeFromBodyListsParent(int p);
    void removeEmptyBodyPairContacts();
    int updateBodyPairContacts();
    int pullBodies();
    int pushBodies();
    int ensureStore(int need);
    int copyContacts(const DContacts& S, const std::vector<int>& si, DContacts& D, const std::vector<int>& di, int mode);
    int newSlot();
    int toInternal(int p);
    int ensureSweep(int need);
    void nextLayer(std::vector<int>& layer, std::vector<int>& ordered);
    int singleSweep(double dt);
    int metrics(const std::vector<int>& a, const std::vector<int>& b, const std::vector<int>& mode, std::vector<double>& out);
    int accumulateForUnmerging();
    int pullStates(bool internalToo);
    int newCollectionSlot();
    void collApplyVelocitiesTo(int c, int b);
    void collUpdateState(int c, int b);
    void collUpdateBB(int c, int b);
    void setBB(int c, amd::v3 mn, amd::v3 mx);
    void collUpdateBBAll(int c);
    void collAddInternal(int c, int b);
    void collInertiaRestInvert(int c);
    void rotInertia(int b);
    void collBodiesTransforms(int c);
    void collAddBody(int c, int b);
    void collAddBodies(int c, const std::vector<int>& bs);
    void collAddCollection(int c, int o);
    void freeCollection(int c);
    int newCollection(int b1, int b2);
    void collRemoveBodies(int c, const std::vector<int>& rm);
    void collAddBPCs(int p);
    void collFillInternal(int c);
    int collAddIncomplete(int body, std::vector<int>& removal);
    void collUnmergeBody(int c, int b);
    bool checkMergeCondition(int p);
    int merge();
    void buildNeighbor(int b, OSetI& sub, OSetI& handled);
    int unmergeSelected(int coll, OSetI& sel, std::vector<int>& newBodies, bool& removeCollection);
    int unmerge();
    int clearBodyPairContacts();
    int accumulateForMerging();
    int uploadExternalFlags();
    int appendFromStore(const std::vector<int>& slots, std::vector<int>& newIdx);
    int ensurePairsKeep(int need);
    int flushAppendedPairs();
    void advVel(double dt);
    void advPos(double dt);
    int sleepDecay();
    int getTopology(int* items, int* itemOff, int capItems, int* nTop, int* nItems);
    int setBatch(const am_scene* scenes, int n);
    int stepBatch(double dt);
    int batchSolve(double dt);
    int batchStats();
    int batchAutotune(double dt);
    int batchColours(int* out);
    int getState(std::vector<uint8_t>& out);
    int mergeTests(std::vector<int>& a, std::vector<int>& b, std::vector<int>& kind, std::vector<int>& result,
                   std::vector<double>& metric);
    int mergingPhase(int ph, double dt);
    int singleSweepOrder(std::vector<int>& refs);
    int singleSweepRefs(const std::vector<int>& refs, double dt);
    bool anyCollection() const;
    int putState(const uint8_t* in, size_t size);
    int batchChain(int* out);
    int* bChain = nullptr;
    int batchLayout(int cap);
    int batchLaunchSweep(int threads, int cap, int iters, float tol, int check, float* lamStart, const float* lamAlt,
                         int* fall, int writeBack, int nGrid, const int* order, int nbMax, cudaStream_t strm);
    int batchSplit(int cap, bool useCluster);
    int batchLaunchCluster(int q, const int* list, int nBig, cudaStream_t strm, int iters, float tol, int check,
                           int writeBack);
    int batchLaunchAll(int threads, int cap, int iters, float tol, int check, float* lamStart, const float* lamAlt,
                       int writeBack);
    int batchClusterScenes() const;
    int batchClusterMaxK() const;
    void batchSceneCtas(int* out) const;
    int learnedInit();
    int ensureFeat(int nc);
    int learnedFeatures(double dt);
    int learnedRecord();
    int learnedPredict(bool tensorCores);
    int learnedPackInference();
    int learnedNormalise();
    int learnedTrain(int epochs, int batch, float lr, float* lastLoss, int normalise);
    int learnedGrad(const float* X, const float* Y, int n, float* grad, float* loss);
    int learnedInfer(const float* X, int n, float* out, int tensorCores);
    int learnedWeights(float* w, const float* in, float* norm, const float* normIn);
    int learnedCollect(int enable, int capacity);
    int learnedInferNoAlloc(const float* X, int n, float* out, int tensorCores);
    std::vector<void*> tmps;
    int* flagStage = nullptr;    // pinned host staging of body flags (getBodies)
    int flagStageCap = 0;
    template <class T>
    int tmpAlloc(T** p, size_t n);
    int tmpFree(int r);
    int putBodies(const am_body_state* in);
    int getContacts(am_contacts* out, int capacity, int* n);
};

// device allocation owned by the context (freed in release())
template <class T>
int Ctx::alloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc((void**)p, sizeof(T) * n) != cudaSuccess) { err = "cudaMalloc failed"; return AM_E_CUDA; }
    allocs.push_back((void*)*p);
    return AM_OK;
}

void launch_put_free(const DBodies& B, int n, const int* parent, const double* x, const double* R, const double* v,
                     const double* w, cudaStream_t s);
const void* pgs_fast_kernel();
const void* pgs_mixed_kernel();
const void* gs_levels_kernel();
const void* batch_sweep_kernel();
int learned_num_params();
int gs_levels(const std::vector<int>& s1, const std::vector<int>& s2, const std::vector<int>& flags,
              std::vector<int>& order, std::vector<int>& levelOff, std::vector<int>& last);
void launch_gs_levels(const DBodies& B, DContacts& C, const int* order, const int* levelOff, int nLevels, int iters,
                      double omega, double comp, double tol, bool early, int fo, double fv, double slide,
                      DCount* dc, int blocks, cudaStream_t s);
void launch_refresh_inertia(const DBodies& B, int n, cudaStream_t s);
void launch_sub_adv_vel(const DBodies& B, const int* top, int ntop, const int* so, const int* si, double dt,
                        cudaStream_t s);

}  // namespace am
