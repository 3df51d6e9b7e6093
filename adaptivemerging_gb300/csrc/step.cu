// step.cu -- body kernels (forces, integration, sleeping) and the context
// that drives one simulation step on the device behind the C ABI.
//
// The context mirrors the reference's call surface: Ctx::step follows
// RigidBodySystem.advanceTime (RigidBodySystem.java:102-185) phase by phase;
// collisionDetection / warmStart / solveLCP / updateInCollections follow the
// CollisionProcessor methods of the same names.  Body state, contacts and
// pairs stay resident in HBM between steps; the host only reads back the
// three sizes (candidate pairs, sub-body pairs, contacts) needed to size the
// next launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "am_ctx.hpp"
#include "am_dev.cuh"
#include "collections.hpp"

namespace am {
using namespace amd;

// ---------------------------------------------------------------------------
// RigidBodySystem.clearBodies + applyGravityForce (RigidBodySystem.java:190-202,
// 276-290) and RigidCollection.clearBodies / applyVelocitiesTo (RigidCollection.java:100-105, 925-937)
__device__ __forceinline__ void apply_vel_to(const DBodies& B, int c, int b) {
    v3 r = sub(ldv(B.x + 3 * b), ldv(B.x + 3 * c));
    v3 wxr = cross(ldv(B.w + 3 * c), r);
    stv(B.v + 3 * b, add(ldv(B.v + 3 * c), wxr));
    stv(B.w + 3 * b, ldv(B.w + 3 * c));
}

__device__ __forceinline__ void clear_body(const DBodies& B, int b) {
    for (int k = 0; k < 3; k++) { B.force[3 * b + k] = 0.0; B.torque[3 * b + k] = 0.0; }
    for (int k = 0; k < 6; k++) B.dv[6 * b + k] = 0.0;
}

__device__ __forceinline__ void gravity(const DBodies& B, int b, v3 g) {
    v3 f = scale(-B.mass[b], g);
    stv(B.force + 3 * b, add(ldv(B.force + 3 * b), f));
}

// mode 0: clearBodies + gravity; mode 1: mergingEvent re-clear of top-level
// bodies + gravity again (RigidBodySystem.java:138-142)
__global__ void k_begin(DBodies B, const int* top, int ntop, const int* so, const int* si, v3 g, int useG,
                        int mode) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int b = top[i];
    clear_body(B, b);
    bool coll = B.flags[b] & F_COLLECTION;
    if (coll && mode == 0)
        for (int k = so[b]; k < so[b + 1]; k++) {
            int s = si[k];
            apply_vel_to(B, b, s);
            clear_body(B, s);
        }
    if (useG) {
        gravity(B, b, g);
        if (coll)
            for (int k = so[b]; k < so[b + 1]; k++) gravity(B, si[k], g);
    }
}

// RigidBody.advanceVelocities (RigidBody.java:409-417)
__device__ void adv_vel(const DBodies& B, int b, double dt) {
    v3 v = scaleadd(dt * B.minv[b], ldv(B.force + 3 * b), ldv(B.v + 3 * b));
    v = add(v, ldv(B.dv + 6 * b));
    stv(B.v + 3 * b, v);
    v3 dw = mxv(ldm(B.jinv + 9 * b), ldv(B.torque + 3 * b));
    dw.x *= dt; dw.y *= dt; dw.z *= dt;
    v3 w = add(ldv(B.w + 3 * b), dw);
    w = add(w, ldv(B.dv + 6 * b + 3));
    stv(B.w + 3 * b, w);
}

// RigidBody.advancePositions + expRodrigues + updateRotationalInertiaFromTransformation
// + updateBBW (RigidBody.java:311-441)
__device__ void adv_pos(const DBodies& B, int b, double dt) {
    v3 x = scaleadd(dt, ldv(B.v + 3 * b), ldv(B.x + 3 * b));
    stv(B.x + 3 * b, x);
    v3 om = ldv(B.w + 3 * b);
    double t = length(om) * dt;
    v3 w = om;
    normalize(w);
    m3 R = ldm(B.R + 9 * b);
    if (t > 1e-8) {
        double s, c;
        det_sincos(t, &s, &c);
        double c1 = 1 - c;
        m3 dR;
        dR.m[0] = c + w.x * w.x * c1;
        dR.m[3] = w.z * s + w.x * w.y * c1;
        dR.m[6] = -w.y * s + w.x * w.z * c1;
        dR.m[1] = -w.z * s + w.x * w.y * c1;
        dR.m[4] = c + w.y * w.y * c1;
        dR.m[7] = w.x * s + w.y * w.z * c1;
        dR.m[2] = w.y * s + w.x * w.z * c1;
        dR.m[5] = -w.x * s + w.y * w.z * c1;
        dR.m[8] = c + w.z * w.z * c1;
        R = normalizeCP(mmul(dR, R));
        stm(B.R + 9 * b, R);
    }
    if (!(B.flags[b] & F_PINNED)) {
        stm(B.M + 9 * b, rm0rt(R, ldm(B.M0 + 9 * b)));
        stm(B.jinv + 9 * b, rm0rt(R, ldm(B.jinv0 + 9 * b)));
    }
}

// RigidCollection.updateBodiesPositionAndTransformations (RigidCollection.java:898-909)
__device__ void coll_update_subs(const DBodies& B, int c, const int* so, const int* si) {
    m3 Rc = ldm(B.R + 9 * c);
    v3 xc = ldv(B.x + 3 * c);
    bool pinned = B.flags[c] & F_PINNED;
    for (int k = so[c]; k < so[c + 1]; k++) {
        int b = si[k];
        m3 Rb = ldm(B.B2C + 12 * b);
        v3 tb = ldv(B.B2C + 12 * b + 9);
        v3 xb = add(mxv(Rc, tb), xc);      // RigidTransform3D.mult(A, B)
        m3 R = mmul(Rc, Rb);
        stv(B.x + 3 * b, xb);
        stm(B.R + 9 * b, R);
        if (!pinned) {
            stm(B.jinv + 9 * b, rm0rt(R, ldm(B.jinv0 + 9 * b)));
            stm(B.M + 9 * b, rm0rt(R, ldm(B.M0 + 9 * b)));
        }
    }
}

__global__ void k_adv_vel(DBodies B, const int* top, int ntop, const int* so, const int* si, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int b = top[i];
    int f = B.flags[b];
    if ((f & F_PINNED) || (f & F_SLEEPING)) return;
    adv_vel(B, b, dt);
    if (f & F_COLLECTION)   // RigidCollection.advanceVelocities -> applyVelocitiesToBodies
        for (int k = so[b]; k < so[b + 1]; k++) apply_vel_to(B, b, si[k]);
}

__global__ void k_adv_pos(DBodies B, const int* top, int ntop, const int* so, const int* si, double dt,
                          DCount* dc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int b = top[i];
    int f = B.flags[b];
    if ((f & F_PINNED) || (f & F_SLEEPING)) return;
    // a non-finite velocity (from non-finite inputs or a diverged solve) is
    // reported as AM_E_NONFINITE; the arithmetic itself is left as it is
    bool fin = true;
    for (int k = 0; k < 3; k++) fin = fin && isfinite(B.v[3 * b + k]) && isfinite(B.w[3 * b + k]);
    if (!fin) atomicExch(&dc->error, AM_E_NONFINITE);
    adv_pos(B, b, dt);
    if (f & F_COLLECTION) coll_update_subs(B, b, so, si);
}

// sub-body velocity advance after the single sweep (CollisionProcessor.java:289-299)
__global__ void k_sub_adv_vel(DBodies B, const int* top, int ntop, const int* so, const int* si, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int b = top[i];
    int f = B.flags[b];
    if ((f & F_COLLECTION) && !(f & F_SLEEPING))
        for (int k = so[b]; k < so[b + 1]; k++) {
            int s = si[k];
            if (!(B.flags[s] & F_PINNED)) adv_vel(B, s, dt);
        }
    for (int k = 0; k < 6; k++) B.dv[6 * b + k] = 0.0;
}

void launch_sub_adv_vel(const DBodies& B, const int* top, int ntop, const int* so, const int* si, double dt,
                        cudaStream_t s) {
    if (ntop <= 0) return;
    k_sub_adv_vel<<<(ntop + 127) / 128, 128, 0, s>>>(B, top, ntop, so, si, dt);
    AM_LAUNCHED(1);
}

// MotionMetricProcessor.getLargestVelocityNorm(body) (MotionMetricProcessor.java:64-73)
__device__ double metric1(const DBodies& B, int b) {
    double largest = 0;
    if (B.type[b] == AM_PLANE) return 0;
    m3 R = ldm(B.R + 9 * b);
    v3 x = ldv(B.x + 3 * b), v = ldv(B.v + 3 * b), w = ldv(B.w + 3 * b);
    for (int k = 0; k < 8; k++) {
        v3 pW = tpoint(R, x, ldv(B.bbB + 24 * b + 3 * k));
        v3 r = cross(w, sub(pW, x));
        largest = jmax(length(add(r, v)), largest);
    }
    return largest;
}

// Sleeping.wake (Sleeping.java:107-139): a body pair with no pinned body wakes
// both of its bodies (and their collections) when either top-level side sleeps.
__global__ void k_wake_mark(DBodies B, DPairs P, int npairs, int* wake) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs || P.count[p] == 0) return;
    int a = P.a[p], b = P.b[p];
    if ((B.flags[a] & F_PINNED) || (B.flags[b] & F_PINNED)) return;
    int ta = B.parent[a] >= 0 ? B.parent[a] : a;
    int tb = B.parent[b] >= 0 ? B.parent[b] : b;
    if ((B.flags[ta] & F_SLEEPING) || (B.flags[tb] & F_SLEEPING)) {
        wake[a] = 1; wake[b] = 1;
        if (ta != a) wake[ta] = 1;
        if (tb != b) wake[tb] = 1;
    }
}

__global__ void k_wake_apply(DBodies B, int n, int* wake) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n || !wake[b]) return;
    wake[b] = 0;
    if (B.flags[b] & F_SLEEPING) { B.flags[b] &= ~F_SLEEPING; B.hist_n[b] = 0; B.hist_h[b] = 0; }
}

// external non-pinned body pairs that survive clearBodyPairContacts keep
// their top-level bodies awake in Sleeping.sleep (Sleeping.java:65-73)
__global__ void k_ext_mark(DBodies B, DPairs P, int npairs, int* ext) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs || !P.keep[p]) return;
    int a = P.a[p], b = P.b[p];
    if ((B.flags[a] & F_PINNED) || (B.flags[b] & F_PINNED)) return;
    ext[B.parent[a] >= 0 ? B.parent[a] : a] = 1;
    ext[B.parent[b] >= 0 ? B.parent[b] : b] = 1;
}

// Sleeping.sleep + accumulate (Sleeping.java:49-98, 155-160) and
// RigidBodySystem.applyViscousDecay (RigidBodySystem.java:428-436)
__global__ void k_sleep_decay(DBodies B, const int* top, int ntop, int* ext, int enable, int accum, double thr,
                              double a1, double a2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntop) return;
    int b = top[i];
    int isExt = ext[b];
    ext[b] = 0;
    if (enable && !(B.flags[b] & F_SLEEPING) && !isExt) {
        double m = metric1(B, b);
        int n = B.hist_n[b], h = B.hist_h[b];
        double* H = B.hist + HIST * b;
        H[(h + n) % HIST] = m;
        if (n < accum) n++;
        else h = (h + 1) % HIST;
        B.hist_n[b] = n; B.hist_h[b] = h;
        bool s = true;
        double prev = 1.79769313486231570e308, eps = 5e-5;
        if (n < accum) s = false;
        else
            for (int k = 0; k < n; k++) {
                double q = H[(h + k) % HIST];
                if (q > prev + eps) { s = false; break; }
                if (q > thr) { s = false; break; }
                prev = q;
            }
        if (s) B.flags[b] |= F_SLEEPING; else B.flags[b] &= ~F_SLEEPING;
    }
    v3 v = ldv(B.v + 3 * b), w = ldv(B.w + 3 * b);
    v.x *= a1; v.y *= a1; v.z *= a1;
    w.x *= a2; w.y *= a2; w.z *= a2;
    stv(B.v + 3 * b, v);
    stv(B.w + 3 * b, w);
}

// am_put_bodies: after x / R / v / omega of free bodies were overwritten from
// the host, refresh the rotated inertia as RigidBody.updateRotationalInertiaFromTransformation does
__global__ void k_refresh_inertia(DBodies B, int n) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n || (B.flags[b] & F_PINNED)) return;
    m3 R = ldm(B.R + 9 * b);
    stm(B.M + 9 * b, rm0rt(R, ldm(B.M0 + 9 * b)));
    stm(B.jinv + 9 * b, rm0rt(R, ldm(B.jinv0 + 9 * b)));
}

void launch_refresh_inertia(const DBodies& B, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_refresh_inertia<<<(n + 127) / 128, 128, 0, s>>>(B, n);
    AM_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
static int g_numSMs = 0;

#define CK(call)                                                                    \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            return AM_E_CUDA;                                                       \
        }                                                                           \
    } while (0)


Ctx::Ctx(const am_params& p) : P(p) {
    cudaGetDevice(&device);
    std::memset(&B, 0, sizeof(B));
    std::memset(&N, 0, sizeof(N));
    std::memset(&C[0], 0, sizeof(DContacts) * 2);
    std::memset(&PR, 0, sizeof(PR));
    std::memset(&H, 0, sizeof(H));
    std::memset(&SC, 0, sizeof(SC));
}

Ctx::~Ctx() { release(); }

void Ctx::release() {
    for (void* q : allocs) cudaFree(q);
    allocs.clear();
    if (dc) cudaFree(dc);
    dc = nullptr;
    if (hc) cudaFreeHost(hc);
    hc = nullptr;
    if (flagStage) cudaFreeHost(flagStage);
    flagStage = nullptr;
    flagStageCap = 0;
    if (hColPin) cudaFreeHost(hColPin);
    hColPin = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    for (int q = 0; q < NPOOL; q++) {
        if (pool[q]) { cudaStreamSynchronize(pool[q]); cudaStreamDestroy(pool[q]); }
        pool[q] = nullptr;
        if (poolJoin[q]) cudaEventDestroy(poolJoin[q]);
        poolJoin[q] = nullptr;
    }
    if (evFork) cudaEventDestroy(evFork);
    evFork = nullptr;
    if (evA && evA != evPh[3]) { cudaEventDestroy(evA); cudaEventDestroy(evB); }
    evA = evB = nullptr;
    for (auto& e : evPh) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    // every device buffer went with `allocs`: forget them and their capacities,
    // so a context given a new scene allocates afresh
    std::memset(&PR, 0, sizeof(PR));
    std::memset(&H, 0, sizeof(H));
    std::memset(&SC, 0, sizeof(SC));
    candA = candB = nullptr;
    candCap = 0;
    Mj = invD = nullptr;
    mjCap = 0;
    mixF = mixU = nullptr;
    mixG = nullptr;
    mixFCap = mixUCap = mixGCap = 0;
    putStage = nullptr;
    putParent = nullptr;
    putStageCap = 0;
    levOrder = levOff = nullptr;
    levCap = 0;
    idxA = idxB = nullptr;
    idxCap = 0;
    metA = metB = metM = nullptr;
    metOut = nullptr;
    metCap = 0;
    pairCls = nullptr;
    broadMask = nullptr;
    broadMaskCap = 0;
    stageD = nullptr;
    stageI = nullptr;
    stageCap = 0;
    bCS = nullptr;
}


int Ctx::allocContacts(DContacts& c, int cap) {
    c.cap = cap;
    int r = 0;
    r |= alloc(&c.b1, cap); r |= alloc(&c.b2, cap); r |= alloc(&c.bv1, cap); r |= alloc(&c.bv2, cap);
    r |= alloc(&c.info, cap); r |= alloc(&c.pair, cap); r |= alloc(&c.state, cap); r |= alloc(&c.fresh, cap);
    r |= alloc(&c.sb1, cap); r |= alloc(&c.sb2, cap);
    r |= alloc(&c.f, 12 * (size_t)cap); r |= alloc(&c.J, 36 * (size_t)cap); r |= alloc(&c.cv, cap);
    r |= alloc(&c.pcv, cap); r |= alloc(&c.lam, 3 * (size_t)cap); r |= alloc(&c.lamw, 3 * (size_t)cap);
    r |= alloc(&c.bD, 6 * (size_t)cap); r |= alloc(&c.Ia, 9 * (size_t)cap); r |= alloc(&c.Ib, 9 * (size_t)cap);
    return r ? AM_E_CUDA : AM_OK;
}

// Grow the current contact buffer (the previous one keeps its capacity and data).
int Ctx::ensureContacts(int need) {
    DContacts& c = C[cur];
    if (need <= c.cap) return AM_OK;
    int cap = std::max(need + need / 2, 1024);
    DContacts nc;
    std::memset(&nc, 0, sizeof(nc));
    int r = allocContacts(nc, cap);
    if (r) return r;
    c = nc;   // old allocation stays in `allocs` until release (no device frees in the step)
    return AM_OK;
}

int Ctx::ensurePairs(int need) {
    if (need <= PR.cap) return AM_OK;
    int cap = std::max(need + need / 2, 1024);
    DPairs np;
    np.cap = cap;
    int r = 0;
    r |= alloc(&np.a, cap); r |= alloc(&np.b, cap); r |= alloc(&np.count, cap); r |= alloc(&np.off, cap + 1);
    r |= alloc(&np.keep, cap); r |= alloc(&np.perm, cap);
    r |= alloc(&colourOf, cap); r |= alloc(&groupOrder, cap);
    if (r) return AM_E_CUDA;
    PR = np;
    return ensureScratch(cap + 1);
}

int Ctx::ensureScratch(int need) {
    if (need <= SC.cap_int) return AM_OK;
    int cap = std::max(need + need / 2, 4096);
    Scratch s;
    s.cap_int = cap;
    // the scan's two levels of block sums (n up to 2^30; callers scan at most cap entries)
    s.cap_block = std::max(4096, cap / 1024 + 2 + 1024);
    int r = alloc(&s.tmp, cap) | alloc(&s.tmp2, cap) | alloc(&s.block, s.cap_block);
    if (r) return AM_E_CUDA;
    SC = s;
    return AM_OK;
}

int Ctx::ensureCand(int need) {
    if (need <= candCap) return AM_OK;
    int cap = std::max(need + need / 2, 1024);
    int r = alloc(&candA, cap) | alloc(&candB, cap);
    if (r) return AM_E_CUDA;
    candCap = cap;
    return ensureScratch(cap + 1);
}

// ---- scene upload ------------------------------------------------------------
int Ctx::setScene(const am_scene& s) {
    release();
    kin.clear();   // prescribed motions name bodies of the previous scene
    kinSteps = 0;
    nScenes = 0;
    topEnd = nullptr;
    bRecCap = bPairCap = 0;
    batchThreads = 0;
    batchThreadsUser = 0;
    batchTunedContacts = 0;
    batchCap = 0;
    batchCapUser = 0;
    bSceneOrder = nullptr;
    // device buffers of the learned start went with release()
    lW = lG = lM = lV = lNorm = lBias = lLoss = nullptr;
    lWb = nullptr;
    lX = lY = lDX = lDY = lZ1 = lZ2 = lYh = nullptr;
    lXN = lA1 = lA2 = lD1 = lD2 = lDYb = nullptr;
    lKeep = lPos = lIdx = nullptr;
    lFeatCap = lDcap = lDn = lTrainCap = lIdxCap = 0;
    lCollect = lUse = 0;
    if (s.n_bodies <= 0) { err = "empty scene"; return AM_E_ARG; }
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaMalloc((void**)&dc, sizeof(DCount)));
    CK(cudaMallocHost((void**)&hc, sizeof(DCount)));
    CK(cudaMallocHost((void**)&hColPin, sizeof(int) * (MAXC + 1)));
    CK(cudaMemsetAsync(dc, 0, sizeof(DCount), stream));
    if (!g_numSMs) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_numSMs, cudaDevAttrMultiProcessorCount, dev);
    }
    nScene = s.n_bodies;
    narrowStageable = true;   // boxes, planes and single spheres: at most 8 contacts per pair
    for (int i = 0; i < s.n_bodies; i++)
        if (s.body_root[i] >= 0 && s.node_nchild[s.body_root[i]] > 0) narrowStageable = false;
    host.init(s, P);
    int cap = host.cap;
    B.n = cap;
    int r = 0;
    r |= alloc(&B.type, cap); r |= alloc(&B.flags, cap); r |= alloc(&B.parent, cap); r |= alloc(&B.root, cap);
    r |= alloc(&B.x, 3 * cap); r |= alloc(&B.R, 9 * cap); r |= alloc(&B.v, 3 * cap); r |= alloc(&B.w, 3 * cap);
    r |= alloc(&B.mass, cap); r |= alloc(&B.minv, cap); r |= alloc(&B.jinv, 9 * cap); r |= alloc(&B.jinv0, 9 * cap);
    r |= alloc(&B.M, 9 * cap); r |= alloc(&B.M0, 9 * cap); r |= alloc(&B.force, 3 * cap);
    r |= alloc(&B.torque, 3 * cap); r |= alloc(&B.dv, 6 * cap); r |= alloc(&B.size, 3 * cap);
    r |= alloc(&B.radius, cap); r |= alloc(&B.friction, cap); r |= alloc(&B.restitution, cap);
    r |= alloc(&B.plane, 4 * cap); r |= alloc(&B.pp, 3 * cap); r |= alloc(&B.bbB, 24 * cap);
    r |= alloc(&B.hist, HIST * cap); r |= alloc(&B.hist_n, cap); r |= alloc(&B.hist_h, cap);
    r |= alloc(&B.bc, cap);
    r |= alloc(&B.B2C, 12 * cap);
    r |= alloc(&top, cap); r |= alloc(&subOff, cap + 1); r |= alloc(&subIds, cap);
    r |= alloc(&rowCount, cap + 1); r |= alloc(&rowOff, cap + 1); r |= alloc(&wakeFlag, cap); r |= alloc(&extFlag, cap);
    // colouring: a 64-bit priority, then a mask of Ctx::MAXC colours (4 words) per body
    r |= alloc(&bodyMax, 10 * (size_t)cap);
    r |= alloc(&colourCnt, MAXC + 1); r |= alloc(&colourOff, MAXC + 2); r |= alloc(&colourFill, MAXC + 1);
    N.n = s.n_nodes;
    r |= alloc(&N.cB, 3 * (size_t)N.n); r |= alloc(&N.cW, 3 * (size_t)N.n); r |= alloc(&N.r, N.n);
    r |= alloc(&N.child0, N.n); r |= alloc(&N.nchild, N.n); r |= alloc(&N.body, N.n);
    if (r) return AM_E_CUDA;
    CK(cudaMemsetAsync(wakeFlag, 0, sizeof(int) * cap, stream));
    CK(cudaMemsetAsync(extFlag, 0, sizeof(int) * cap, stream));
    CK(cudaMemsetAsync(B.hist_n, 0, sizeof(int) * cap, stream));
    CK(cudaMemsetAsync(B.hist_h, 0, sizeof(int) * cap, stream));
    CK(cudaMemsetAsync(B.dv, 0, sizeof(double) * 6 * cap, stream));
    CK(cudaMemsetAsync(B.force, 0, sizeof(double) * 3 * cap, stream));
    CK(cudaMemsetAsync(B.torque, 0, sizeof(double) * 3 * cap, stream));
    // static per-node data
    std::vector<int> nbody(N.n, 0);
    for (int i = 0; i < s.n_bodies; i++) {
        int r0 = s.body_root[i];
        if (r0 < 0) continue;
        std::vector<int> st{r0};
        while (!st.empty()) {
            int q = st.back(); st.pop_back();
            nbody[q] = i;
            for (int k = 0; k < s.node_nchild[q]; k++) st.push_back(s.node_child0[q] + k);
        }
    }
    if (N.n) {
        CK(cudaMemcpyAsync(N.cB, s.node_c, sizeof(double) * 3 * N.n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(N.r, s.node_r, sizeof(double) * N.n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(N.child0, s.node_child0, sizeof(int) * N.n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(N.nchild, s.node_nchild, sizeof(int) * N.n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(N.body, nbody.data(), sizeof(int) * N.n, cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
    int rr = uploadBodies(true);
    if (rr) return rr;
    cur = 0;
    nContacts = 0;
    nPairs = 0;
    totalSteps = 0;
    mergingEvent = false;
    if (allocContacts(C[0], 1024) || allocContacts(C[1], 1024)) return AM_E_CUDA;
    std::memset(&I, 0, sizeof(I));
    std::memset(&Sw, 0, sizeof(Sw));
    idxCap = metCap = 0;
    M.reset(host.cap);
    devDv.assign(6 * (size_t)host.cap, 0.0);
    mergeEvents = unmergeEvents = 0;
    appended = 0;
    if (alloc(&nbbDev, host.cap)) return AM_E_CUDA;
    CK(cudaMemcpyAsync(nbbDev, host.nbb.data(), sizeof(int) * host.cap, cudaMemcpyHostToDevice, stream));
    H.cap = 0;
    if (ensurePairs(1024) || ensureCand(1024)) return AM_E_CUDA;
    return syncErr();
}

// host mirror -> device (all body slots); `full` also sends static data
int Ctx::uploadBodies(bool full) {
    const HostWorld& h = host;
    int cap = h.cap;
    (void)full;
    CK(cudaMemcpyAsync(B.type, h.type.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.flags, h.flags.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.parent, h.parent.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.root, h.root.data(), sizeof(int) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.x, h.x.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.R, h.R.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.v, h.v.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.w, h.w.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.mass, h.mass.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.minv, h.minv.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.jinv, h.jinv.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.jinv0, h.jinv0.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.M, h.M.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.M0, h.M0.data(), sizeof(double) * 9 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.size, h.size.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.radius, h.radius.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.friction, h.friction.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.restitution, h.restitution.data(), sizeof(double) * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.plane, h.plane.data(), sizeof(double) * 4 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.pp, h.pp.data(), sizeof(double) * 3 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.bbB, h.bbB.data(), sizeof(double) * 24 * cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.B2C, h.B2C.data(), sizeof(double) * 12 * cap, cudaMemcpyHostToDevice, stream));
    return uploadTopology();
}

int Ctx::uploadTopology() {
    const HostWorld& h = host;
    ntop = (int)h.top.size();
    CK(cudaMemcpyAsync(top, h.top.data(), sizeof(int) * ntop, cudaMemcpyHostToDevice, stream));
    std::vector<int> so(h.cap + 1, 0), si;
    for (int b = 0; b < h.cap; b++) {
        so[b] = (int)si.size();
        if (h.flags[b] & F_COLLECTION)
            for (int s : h.subs[b]) si.push_back(s);
    }
    so[h.cap] = (int)si.size();
    nSubIds = (int)si.size();
    CK(cudaMemcpyAsync(subOff, so.data(), sizeof(int) * (h.cap + 1), cudaMemcpyHostToDevice, stream));
    if (!si.empty())
        CK(cudaMemcpyAsync(subIds, si.data(), sizeof(int) * si.size(), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.flags, h.flags.data(), sizeof(int) * h.cap, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(B.parent, h.parent.data(), sizeof(int) * h.cap, cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    return AM_OK;
}

int Ctx::syncErr() {
    cudaError_t e = cudaStreamSynchronize(stream);
    // a launch refused for its configuration is not sticky and leaves the
    // stream clean; it shows only in the last-error slot
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("CUDA: ") + cudaGetErrorString(e); return AM_E_CUDA; }
    return AM_OK;
}

int Ctx::readCounts() {
    cudaError_t e = cudaMemcpyAsync(hc, dc, sizeof(DCount), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { err = std::string("CUDA: ") + cudaGetErrorString(e); return AM_E_CUDA; }
    if (hc->error) {
        int code = hc->error;
        err = code == AM_E_TIMEOUT     ? "device wait gave up (grid barrier)"
              : code == AM_E_NONFINITE ? "a body velocity became NaN or infinite"
                                       : "device capacity exceeded (tree stack, colours or staging chunks)";
        cudaMemsetAsync(&dc->error, 0, sizeof(int), stream);
        return code;
    }
    return AM_OK;
}

// ---- phases ------------------------------------------------------------------
void Ctx::gravityDir(double g[3]) const {
    double th = P.gravity_angle / 180.0 * M_PI;
    g[0] = P.gravity_amount * std::cos(th);
    g[1] = P.gravity_amount * std::sin(th);
    g[2] = 0;
}

// Pinned bodies with a prescribed oscillation (am_set_kinematic): at the start
// of the n-th step since the call, x = x0 + axis * (amp * sin(w n dt)) and
// v = axis * ((amp * w) * cos(w n dt)), evaluated on the host with the same
// sine and cosine as the integrator's rotation update, and written to the
// device with one small launch
struct KinSet {
    int n;
    int body[Ctx::MAXKIN];
    double x[Ctx::MAXKIN][3], v[Ctx::MAXKIN][3];
};
__global__ void k_set_kin(DBodies B, KinSet K) {
    int i = threadIdx.x;
    if (i >= K.n) return;
    const int b = K.body[i];
    for (int k = 0; k < 3; k++) {
        B.x[3 * b + k] = K.x[i][k];
        B.v[3 * b + k] = K.v[i][k];
    }
}

// am_put_bodies with collections: rows of free bodies (parent < 0) from the
// staged arrays (any of them may be absent)
__global__ void k_put_free(DBodies B, int n, const int* parent, const double* x, const double* R, const double* v,
                           const double* w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || parent[i] >= 0) return;
    for (int k = 0; k < 3; k++) {
        if (x) B.x[3 * i + k] = x[3 * i + k];
        if (v) B.v[3 * i + k] = v[3 * i + k];
        if (w) B.w[3 * i + k] = w[3 * i + k];
    }
    if (R)
        for (int k = 0; k < 9; k++) B.R[9 * i + k] = R[9 * i + k];
}

void launch_put_free(const DBodies& B, int n, const int* parent, const double* x, const double* R, const double* v,
                     const double* w, cudaStream_t s) {
    if (n <= 0) return;
    k_put_free<<<(n + 255) / 256, 256, 0, s>>>(B, n, parent, x, R, v, w);
    AM_LAUNCHED(1);
}

void Ctx::applyKinematic() {
    if (kin.empty()) return;
    KinSet K{};
    K.n = (int)kin.size();
    for (int i = 0; i < K.n; i++) {
        const Kinematic& q = kin[i];
        const double t = (double)kinSteps * q.dt;
        double sn, cs;
        amd::det_sincos(q.omega * t, &sn, &cs);
        K.body[i] = q.body;
        for (int k = 0; k < 3; k++) {
            K.x[i][k] = q.x0[k] + q.axis[k] * (q.amp * sn);
            K.v[i][k] = q.axis[k] * ((q.amp * q.omega) * cs);
        }
    }
    k_set_kin<<<1, 32, 0, stream>>>(B, K);
    AM_LAUNCHED(1);
    kinSteps++;
}

int Ctx::beginStep(int mode) {
    if (mode == 0) applyKinematic();
    double g[3];
    gravityDir(g);
    if (ntop > 0) {
        k_begin<<<(ntop + 127) / 128, 128, 0, stream>>>(B, top, ntop, subOff, subIds, mk(g[0], g[1], g[2]),
                                                        P.use_gravity, mode);
        AM_LAUNCHED(1);
    }
    return AM_OK;
}

// CollisionProcessor.updateContactsMap + collisionDetection (CollisionProcessor.java:91-102, 443-448)
int Ctx::collisionDetection() {
    cur ^= 1;                    // previous contacts become the warm-start donors
    nPrev = nContacts;
    launch_bv_update(B, N, stream);
    int r = ensureCand(1);
    if (r) return r;
    // hit masks of the count pass, reused by the emit pass (when they fit 256 MB)
    unsigned* masks = nullptr;
    int mw = 0;
    if (ntop >= 2) {
        const int rowMax = nScenes > 0 ? maxSceneBodies : ntop;
        mw = (rowMax + 31) / 32;
        size_t need = (size_t)ntop * (size_t)mw;
        if (need * sizeof(unsigned) <= (size_t)256 << 20) {
            if (need > broadMaskCap) {
                if (alloc(&broadMask, need)) return AM_E_CUDA;
                broadMaskCap = need;
            }
            masks = broadMask;
        } else {
            mw = 0;
        }
    }
    if ((r = ensureScratch(ntop + 1))) return r;   // the rows' scan
    launch_broadphase(B, N, top, ntop, nullptr, nullptr, 0, rowCount, rowOff, SC, dc, stream, topEnd, masks, mw);
    if ((r = readCounts())) return r;
    int ncand = hc->n_cand;
    if ((r = ensureCand(ncand))) return r;
    if (ntop >= 2 && ncand > 0) {
        launch_broadphase(B, N, top, ntop, candA, candB, candCap, rowCount, rowOff, SC, dc, stream, topEnd, masks,
                          mw);
    }
    if ((r = ensureScratch(ncand + 1))) return r;
    // the expansion's scan leaves the pair count in dc->n_pairs for the
    // narrow phase.  Without collections every candidate is one pair, so the
    // host knows the count without waiting for it
    int npairs = 0;
    if (nSubIds == 0) {
        npairs = ncand;
        if (npairs > PR.cap && (r = ensurePairs(npairs))) return r;
        launch_expand_pairs(B, subOff, subIds, candA, candB, ncand, PR, SC, dc, stream);
    } else {
        launch_broad_pack_subs(B, N, subIds, nSubIds, stream);   // bounds of collection members for the expansion
        launch_expand_pairs(B, subOff, subIds, candA, candB, ncand, PR, SC, dc, stream);
        if ((r = readCounts())) return r;
        npairs = ncand > 0 ? hc->n_pairs : 0;
        if (npairs > PR.cap) {
            if ((r = ensurePairs(npairs))) return r;
            launch_expand_pairs(B, subOff, subIds, candA, candB, ncand, PR, SC, dc, stream);
        }
    }
    nPairs = npairs;
    // staged narrow phase (colliders run once) when no pair can exceed the
    // staging slots and the staging fits 512 MB; otherwise count, then emit
    double* sd = nullptr;
    int* si = nullptr;
    if (npairs > 0 && narrowStageable) {
        size_t slots = (size_t)npairs * narrow_stage_slots();
        if (slots * (7 * sizeof(double) + 5 * sizeof(int)) <= ((size_t)512 << 20)) {
            if (slots > stageCap) {
                size_t cap = slots + slots / 2;
                if (alloc(&stageD, 7 * cap) || alloc(&stageI, 5 * cap)) return AM_E_CUDA;
                stageCap = cap;
            }
            sd = stageD;
            si = stageI;
        }
    }
    if (npairs > 0) {
        if (!pairCls && alloc(&pairCls, 16)) return AM_E_CUDA;
        launch_pair_order(B, PR, npairs, pairCls, stream);
        if (sd) cudaMemsetAsync(&dc->stage_ovf, 0, sizeof(int), stream);
        launch_narrow(B, N, PR, C[cur], SC, dc, false, stream, sd, si, &dc->stage_ovf);
        if ((r = ensureScratch(npairs + 1))) return r;
        launch_scan(PR.count, PR.off, npairs, SC, &dc->n_contacts, stream);
        if ((r = readCounts())) return r;
        nContacts = hc->n_contacts;
        if (sd && hc->stage_ovf) {   // a pair kept more contacts than staged: emit pass
            sd = nullptr;
            si = nullptr;
        }
    } else {
        nContacts = 0;
    }
    if ((r = ensureContacts(nContacts))) return r;
    if (nContacts > 0) launch_narrow(B, N, PR, C[cur], SC, dc, true, stream, sd, si, nullptr);
    return AM_OK;
}

// CollisionProcessor.warmStart(false)
int Ctx::warmStart() {
    if (nPairs <= 0) return AM_OK;
    int need = 1;
    while (need < 2 * std::max(nPrev, 1)) need <<= 1;
    if (need > H.cap) {
        int r = alloc(&H.slot, need);
        if (r) return r;
        H.cap = need;
    }
    launch_ws_build(C[cur ^ 1], nPrev, H, stream);
    launch_warm_start(B, C[cur], C[cur ^ 1], H, PR, nPairs, nPrev, stream);
    return AM_OK;
}

int Ctx::wake() {
    if (!P.enable_sleeping || nPairs <= 0) return AM_OK;
    k_wake_mark<<<(nPairs + 255) / 256, 256, 0, stream>>>(B, PR, nPairs, wakeFlag);
    AM_LAUNCHED(1);
    k_wake_apply<<<(host.cap + 255) / 256, 256, 0, stream>>>(B, host.cap, wakeFlag);
    AM_LAUNCHED(1);
    return AM_OK;
}

int Ctx::runPGS(int nc, const int* order, int iters, bool inColl, double dt, bool redoWarm) {
    if (nc <= 0) { stats.sweeps = 0; stats.last_change = 0; return AM_OK; }
    double comp = P.enable_compliance ? P.compliance : 0.;
    DContacts& c = C[cur];
    launch_solve_prep(B, c, nc, dt, P.feedback_stiffness, inColl, P.restitution_override, P.restitution,
                      redoWarm ? 1 : 0, stream);
    bool timed = !inColl;
    if (timed) {
        if (!evA) { cudaEventCreate(&evA); cudaEventCreate(&evB); }
        cudaEventRecord(evA, stream);
    }
    if (P.solver_order == AM_ORDER_REFERENCE || inColl) {
        (void)order;
        int r = exactSweep(c, nc, iters, inColl);
        if (r) return r;
    } else {
        colour_groups(B, c, PR, nPairs, colourOf, colourCnt, colourOff, colourFill, groupOrder, MAXC,
                      (unsigned long long*)bodyMax, host.cap, dc, SC, stream);
        // the colour offsets come back with the counts (one wait)
        cudaMemcpyAsync(hColPin, colourOff, sizeof(int) * (MAXC + 1), cudaMemcpyDeviceToHost, stream);
        int r = readCounts();
        if (r) return r;
        int ncol = hc->n_colours;
        const bool mixed = P.solver_order == AM_ORDER_MIXED;
        if (!coopBlocks) {   // both coloured kernels: 128 threads, at most 4 blocks per SM
            int per = 0, perM = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pgs_fast_kernel(), 128, 0);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perM, pgs_mixed_kernel(), 128, 0);
            coopBlocks = std::max(1, std::min(std::min(per, perM), 4)) * g_numSMs;
        }
        if (nc > mjCap) {
            int cap2 = std::max(nc + nc / 2, 1024);
            if (alloc(&Mj, 36 * (size_t)cap2) || alloc(&invD, (size_t)pgs_fast_krows() * cap2)) return AM_E_CUDA;
            mjCap = cap2;
        }
        // 8 half-warp groups per block; enough blocks for every group of the
        // largest colour (more blocks only make the grid barriers slower)
        hColOff.assign(hColPin, hColPin + ncol + 1);
        if (ncol == 0) hColOff[0] = 0;
        int widest = 0;
        for (int k = 0; k < ncol; k++) widest = std::max(widest, hColOff[k + 1] - hColOff[k]);
        int blocks = std::min(coopBlocks, std::max(1, (widest + 7) / 8));
        if (mixed) {
            if (mjCap > mixFCap) {
                if (alloc(&mixF, (size_t)pgs_mixed_frows() * mjCap)) return AM_E_CUDA;
                mixFCap = mjCap;
            }
            if (host.cap > mixUCap) {
                if (alloc(&mixU, 14 * (size_t)host.cap)) return AM_E_CUDA;   // body data (8) and corrections (6)
                mixUCap = host.cap;
            }
            const int ng = hColOff[ncol];
            if (ng > mixGCap) {
                int cap2 = std::max(ng + ng / 2, 256);
                if (alloc(&mixG, 4 * (size_t)cap2)) return AM_E_CUDA;
                mixGCap = cap2;
            }
            const int mblocks = pgs_mixed_grid_blocks(widest, coopBlocks);
            int form = pgs_mixed_mode(hColOff, mblocks, host.cap, nc);
            if (mixedForm >= 0) form = pgs_mixed_fits(mixedForm, hColOff, host.cap, nc) ? mixedForm : form;
            mixedLastForm = form;
            const int refine = mixedRefine > 0 ? mixedRefine : (solveCheck > 0 ? solveCheck : 100);
            if (timed) cudaEventRecord(evA, stream);
            // refined every `refine` sweeps and at every residual check
            launch_pgs_mixed(B, c, PR, groupOrder, colourOff, ncol, nc, iters, P.omega, comp, P.tolerance, !inColl,
                             P.friction_override, P.friction, P.sliding_threshold, Mj, invD, mixF, mixU,
                             mixU + 8 * (size_t)host.cap, reinterpret_cast<int4*>(mixG), ng, host.cap, mjCap,
                             dc, mblocks, form, stream, inColl ? 0.0 : solveTol, inColl ? 0 : solveCheck, refine);
        } else {
            if (timed) cudaEventRecord(evA, stream);   // time the sweep (prep + persistent kernel)
            launch_pgs_fast(B, c, PR, groupOrder, colourOff, ncol, nc, iters, P.omega, comp, P.tolerance, !inColl,
                            P.friction_override, P.friction, P.sliding_threshold, Mj, invD, mjCap, dc, blocks,
                            stream, inColl ? 0.0 : solveTol, inColl ? 0 : solveCheck);
        }
    }
    if (timed) { cudaEventRecord(evB, stream); pgsPending = true; }
    return AM_OK;
}

// PGS in list order, bit-exact, level scheduled (gs_exact.cu): the levels come
// from the contacts' solve bodies, computed here on the host
int Ctx::exactSweep(DContacts& buf, int n, int iters, bool inColl) {
    hS1.resize(n);
    hS2.resize(n);
    cudaMemcpyAsync(hS1.data(), buf.b1, sizeof(int) * n, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(hS2.data(), buf.b2, sizeof(int) * n, cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    if (!inColl)
        for (int i = 0; i < n; i++) {
            if (host.parent[hS1[i]] >= 0) hS1[i] = host.parent[hS1[i]];
            if (host.parent[hS2[i]] >= 0) hS2[i] = host.parent[hS2[i]];
        }
    hLast.assign(host.cap, 0);
    int nL = gs_levels(hS1, hS2, host.flags, hOrder, hLevOff, hLast);
    if (n > levCap || nL + 1 > levCap) {
        int cap = std::max(2 * std::max(n, nL + 1), 4096);
        if (alloc(&levOrder, cap) || alloc(&levOff, cap)) return AM_E_CUDA;
        levCap = cap;
    }
    int width = 0;
    for (int L = 0; L < nL; L++) width = std::max(width, hLevOff[L + 1] - hLevOff[L]);
    cudaMemcpyAsync(levOrder, hOrder.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(levOff, hLevOff.data(), sizeof(int) * (nL + 1), cudaMemcpyHostToDevice, stream);
    if (!gsBlocksMax) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gs_levels_kernel(), 128, 0);
        gsBlocksMax = std::max(1, per) * g_numSMs;
    }
    // four warps (contacts) per block: one per SM sub-partition's FP64 pipe
    int blocks = std::min(gsBlocksMax, std::max(1, (width + 3) / 4));
    double comp = P.enable_compliance ? P.compliance : 0.;
    launch_gs_levels(B, buf, levOrder, levOff, nL, iters, P.omega, comp, P.tolerance, !inColl, P.friction_override,
                     P.friction, P.sliding_threshold, dc, blocks, stream);
    return AM_OK;
}

// after a synchronising read: fold the timed PGS launch into the counters
void Ctx::foldTiming() {
    if (!pgsPending) return;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, evA, evB) == cudaSuccess) {
        perf.pgs_ms += ms;
        perf.pgs_launches += 1;
        perf.contact_sweeps += (long long)nContacts * (long long)hc->sweeps;
    }
    pgsPending = false;
}

// CollisionProcessor.solveLCP (+ the redoWarmStart that precedes it)
int Ctx::solveLCP(double dt, bool redoWarm) {
    int r = runPGS(nContacts, nullptr, P.iterations, false, dt, redoWarm);
    if (r) return r;
    double comp = P.enable_compliance ? P.compliance : 0.;
    launch_residual(B, C[cur], nContacts, comp, P.friction_override, P.friction, dc, stream);
    return AM_OK;
}

void Ctx::advVel(double dt) {
    if (ntop <= 0) return;
    k_adv_vel<<<(ntop + 127) / 128, 128, 0, stream>>>(B, top, ntop, subOff, subIds, dt);
    AM_LAUNCHED(1);
}

void Ctx::advPos(double dt) {
    if (ntop <= 0) return;
    k_adv_pos<<<(ntop + 127) / 128, 128, 0, stream>>>(B, top, ntop, subOff, subIds, dt, dc);
    AM_LAUNCHED(1);
}

int Ctx::sleepDecay() {
    if (ntop <= 0) return AM_OK;
    k_sleep_decay<<<(ntop + 127) / 128, 128, 0, stream>>>(B, top, ntop, extFlag, P.enable_sleeping,
                                                          P.sleep_step_accum, P.sleep_threshold,
                                                          P.viscous_linear, P.viscous_angular);
    AM_LAUNCHED(1);
    return AM_OK;
}

// clearBodyPairContacts, advanceBodiesVelocities / Positions, sleep, viscous
// decay of the step without merging (pairs are this step's contact runs)
int Ctx::finishStep(double dt) {
    launch_bpc_keep(C[cur], PR, nPairs, stream);
    advVel(dt);
    advPos(dt);
    if (nPairs > 0) {
        k_ext_mark<<<(nPairs + 255) / 256, 256, 0, stream>>>(B, PR, nPairs, extFlag);
        AM_LAUNCHED(1);
    }
    return sleepDecay();
}

int Ctx::step(double dt) {
    totalSteps++;
    int r;
    for (double& v : phase) v = 0.;
    const double t0 = phaseNow();
    if (nScenes > 0) r = stepBatch(dt);
    else if (host.anyMerging()) r = stepWithMerging(dt);
    else r = stepPlain(dt);
    phaseAdd(AM_PHASE_COMPUTE, t0);
    return r;
}

// RigidBodySystem.advanceTime without merging
int Ctx::stepPlain(double dt) {
    int r;
    if ((r = beginStep(0))) return r;
    double t = phaseNow();
    if ((r = collisionDetection())) return r;
    phaseAdd(AM_PHASE_DETECTION, t);
    t = phaseNow();
    if ((r = warmStart())) return r;
    phaseAdd(AM_PHASE_WARMSTART, t);
    if ((r = wake())) return r;
    t = phaseNow();
    if ((r = solveLCP(dt, P.warm_start != 0))) return r;
    phaseAdd(AM_PHASE_LCP_SOLVE, t);
    if ((r = finishStep(dt))) return r;
    if ((r = readCounts())) return r;
    foldTiming();
    perf.steps++;
    return collectStats();
}

int Ctx::collectStats() {
    stats.n_contacts = nContacts;
    stats.sweeps = hc->sweeps;
    stats.last_change = __longlong_as_double_host(hc->maxchg[0]);
    stats.residual_abs = hc->res_abs;
    double lm = hc->lam_max;
    stats.residual_rel = hc->res_abs / (lm > 1 ? lm : 1.0);
    return AM_OK;
}

}  // namespace am
