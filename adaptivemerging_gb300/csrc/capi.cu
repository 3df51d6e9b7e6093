// capi.cu -- the extern "C" entry points declared in include/am.h.
#include <cuda_runtime.h>

#include <cmath>

#include <cstring>
#include <new>
#include <vector>

#include "collections.hpp"

using am::Ctx;

namespace am {

// Body state straight into the caller's arrays (the device arrays hold the
// scene's bodies first, in the same interleaving); the flags go through a
// pinned staging buffer for the sleeping bit.  Pinned caller memory gives
// full-speed copies.
int Ctx::getBodies(am_body_state* o) {
    int n = nScene;
    if (o->x) cudaMemcpyAsync(o->x, B.x, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream);
    if (o->R) cudaMemcpyAsync(o->R, B.R, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, stream);
    if (o->v) cudaMemcpyAsync(o->v, B.v, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream);
    if (o->omega) cudaMemcpyAsync(o->omega, B.w, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream);
    if (o->parent) cudaMemcpyAsync(o->parent, B.parent, sizeof(int) * n, cudaMemcpyDeviceToHost, stream);
    if (o->sleeping) {
        if (n > flagStageCap) {
            if (flagStage) cudaFreeHost(flagStage);
            flagStage = nullptr;
            flagStageCap = 0;
            if (cudaMallocHost((void**)&flagStage, sizeof(int) * n) != cudaSuccess) {
                err = "cudaMallocHost failed";
                return AM_E_CUDA;
            }
            flagStageCap = n;
        }
        cudaMemcpyAsync(flagStage, B.flags, sizeof(int) * n, cudaMemcpyDeviceToHost, stream);
    }
    int r = syncErr();
    if (r) return r;
    if (o->sleeping)
        for (int i = 0; i < n; i++) o->sleeping[i] = (flagStage[i] & F_SLEEPING) ? 1 : 0;
    return AM_OK;
}

// Host-owned state: overwrite x / R / v / omega of the scene bodies that are
// free top-level bodies (bodies inside a collection follow their collection).
// The arrays are expected in pinned host memory for full-speed copies.
int Ctx::putBodies(const am_body_state* in) {
    int n = nScene;
    bool anyColl = false;
    for (int i = 0; i < n; i++) if (host.parent[i] >= 0) { anyColl = true; break; }
    if (!anyColl) {
        if (in->x) cudaMemcpyAsync(B.x, in->x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream);
        if (in->R) cudaMemcpyAsync(B.R, in->R, sizeof(double) * 9 * n, cudaMemcpyHostToDevice, stream);
        if (in->v) cudaMemcpyAsync(B.v, in->v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream);
        if (in->omega) cudaMemcpyAsync(B.w, in->omega, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream);
    } else {
        // bodies inside collections keep the state their collection gives
        // them: the whole arrays go to a staging buffer and one kernel copies
        // the free bodies' rows
        if (putStageCap < 18 * (size_t)n) {
            if (alloc(&putStage, 18 * (size_t)n)) return AM_E_CUDA;
            putStageCap = 18 * (size_t)n;
        }
        if (!putParent) {
            if (alloc(&putParent, (size_t)n)) return AM_E_CUDA;
        }
        cudaMemcpyAsync(putParent, host.parent.data(), sizeof(int) * n, cudaMemcpyHostToDevice, stream);
        double* st[4] = {nullptr, nullptr, nullptr, nullptr};
        const double* src[4] = {in->x, in->R, in->v, in->omega};
        const int w[4] = {3, 9, 3, 3};
        size_t off = 0;
        for (int k = 0; k < 4; k++) {
            if (src[k]) {
                st[k] = putStage + off;
                cudaMemcpyAsync(st[k], src[k], sizeof(double) * w[k] * n, cudaMemcpyHostToDevice, stream);
            }
            off += (size_t)w[k] * n;
        }
        launch_put_free(B, n, putParent, st[0], st[1], st[2], st[3], stream);
    }
    if (in->R) launch_refresh_inertia(B, n, stream);
    return syncErr();
}

int Ctx::getContacts(am_contacts* o, int capacity, int* n) {
    *n = nContacts;
    if (capacity < nContacts) return AM_E_CAPACITY;
    int nc = nContacts;
    if (nc == 0) return AM_OK;
    const DContacts& c = C[cur];
    int cap = c.cap;
    auto geti = [&](int* dst, const int* src) {
        if (dst) cudaMemcpyAsync(dst, src, sizeof(int) * nc, cudaMemcpyDeviceToHost, stream);
    };
    geti(o->body1, c.b1); geti(o->body2, c.b2); geti(o->bv1, c.bv1); geti(o->bv2, c.bv2);
    geti(o->info, c.info); geti(o->state, c.state); geti(o->fresh, c.fresh);
    std::vector<double> f(12 * (size_t)cap), J(36 * (size_t)cap), cv(cap), pcv(cap), lam(3 * (size_t)cap),
        bD(6 * (size_t)cap);
    cudaMemcpyAsync(f.data(), c.f, sizeof(double) * 12 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(J.data(), c.J, sizeof(double) * 36 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(cv.data(), c.cv, sizeof(double) * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(pcv.data(), c.pcv, sizeof(double) * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(lam.data(), c.lam, sizeof(double) * 3 * cap, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(bD.data(), c.bD, sizeof(double) * 6 * cap, cudaMemcpyDeviceToHost, stream);
    int r = syncErr();
    if (r) return r;
    for (int i = 0; i < nc; i++) {
        if (o->frame) for (int k = 0; k < 12; k++) o->frame[12 * i + k] = f[(size_t)k * cap + i];
        if (o->jac) for (int k = 0; k < 36; k++) o->jac[36 * i + k] = J[(size_t)k * cap + i];
        if (o->violation) { o->violation[2 * i] = cv[i]; o->violation[2 * i + 1] = pcv[i]; }
        if (o->lambda) for (int k = 0; k < 3; k++) o->lambda[3 * i + k] = lam[(size_t)k * cap + i];
        if (o->bD) for (int k = 0; k < 6; k++) o->bD[6 * i + k] = bD[(size_t)k * cap + i];
    }
    return AM_OK;
}

}  // namespace am

extern "C" {

void am_params_default(am_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->iterations = 30; p->tolerance = 1e-5; p->omega = 1.0; p->iterations_in_collection = 1;
    p->feedback_stiffness = 0.5; p->enable_compliance = 1; p->compliance = 1e-3;
    p->restitution_override = 0; p->restitution = 0.5; p->friction_override = 0; p->friction = 0.1;
    p->warm_start = 1; p->use_gravity = 1; p->gravity_amount = 1.0; p->gravity_angle = 90.0;
    p->viscous_linear = 1.0; p->viscous_angular = 1.0;
    p->enable_merging = 1; p->enable_merge_pinned = 1; p->enable_merge_cycle = 0;
    p->enable_merge_stable_contact = 1; p->enable_merge_let_it_breathe = 1; p->enable_unmerging = 1;
    p->enable_unmerge_friction = 1; p->enable_unmerge_normal = 1; p->enable_unmerge_relative_motion = 1;
    p->update_contacts_in_collections = 1; p->organize_contacts = 1; p->metric_position_level = 0;
    p->step_accum_merging = 3; p->step_accum_unmerging = 3; p->steps_between_merge_events = 10;
    p->threshold_merge = 1e-2; p->threshold_unmerge = 2e-2; p->threshold_breath = 1e-5;
    p->enable_sleeping = 1; p->sleep_step_accum = 10; p->sleep_threshold = 1e-5;
    p->sliding_threshold = 0.01; p->solver_order = AM_ORDER_REFERENCE;
}

static int check_params(const am_params* p, std::string& err) {
    if (p->enable_merge_cycle) { err = "cycle merge condition is not supported"; return AM_E_ARG; }
    if (p->metric_position_level) { err = "position-level motion metric is not supported"; return AM_E_ARG; }
    if (!p->organize_contacts && p->enable_merging) { err = "organize_contacts = 0 is not supported"; return AM_E_ARG; }
    if (p->sleep_step_accum > am::HIST || p->sleep_step_accum < 0) { err = "sleep_step_accum > 16"; return AM_E_ARG; }
    if (p->iterations < 0) { err = "iterations < 0"; return AM_E_ARG; }
    return AM_OK;
}

int32_t am_create(const am_params* p, void** ctx) {
    if (!p || !ctx) return AM_E_ARG;
    *ctx = nullptr;
    std::string e;
    if (check_params(p, e)) return AM_E_ARG;
    Ctx* c = new (std::nothrow) Ctx(*p);
    if (!c) return AM_E_ARG;
    *ctx = c;
    return AM_OK;
}

int32_t am_destroy(void* ctx) {
    delete (Ctx*)ctx;
    return AM_OK;
}

const char* am_last_error(void* ctx) { return ctx ? ((Ctx*)ctx)->err.c_str() : "null context"; }

int32_t am_set_params(void* ctx, const am_params* p) {
    if (!ctx || !p) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (check_params(p, c->err)) return AM_E_ARG;
    if (p->enable_sleeping && !c->kin.empty()) { c->err = "kinematic bodies need sleeping off"; return AM_E_STATE; }
    c->P = *p;
    c->host.P = &c->P;
    return AM_OK;
}

// A scene is checked on the host before anything reaches the device: the
// tree colliders follow node_child0 / node_nchild, so a child index outside
// the node array would read out of bounds, and a node that is its own
// descendant would never end a traversal.  Every node's children must
// therefore lie after it in the array (as in breadth-first order), which
// also makes every path from a root finite.
static int check_scene(const am_scene& s, std::string& err) {
    if (s.n_bodies < 0 || s.n_nodes < 0) { err = "negative body or node count"; return AM_E_ARG; }
    if (s.n_bodies > 0 && (!s.type || !s.pinned || !s.x || !s.R || !s.v || !s.omega || !s.mass || !s.inertia ||
                           !s.friction || !s.restitution || !s.shape || !s.body_root)) {
        err = "a body array is missing";
        return AM_E_ARG;
    }
    if (s.n_nodes > 0 && (!s.node_c || !s.node_r || !s.node_child0 || !s.node_nchild)) {
        err = "a node array is missing";
        return AM_E_ARG;
    }
    if (s.n_subs != 0) { err = "composite bodies have no device path yet"; return AM_E_ARG; }
    for (int i = 0; i < s.n_bodies; i++) {
        int t = s.type[i];
        if (t == AM_COMPOSITE) { err = "composite bodies have no device path yet"; return AM_E_ARG; }
        if (t < AM_BOX || t > AM_TREE) { err = "unknown body type"; return AM_E_ARG; }
        if ((t == AM_SPHERE || t == AM_TREE) && (s.body_root[i] < 0 || s.body_root[i] >= s.n_nodes)) {
            err = "sphere / tree body without a valid root node";
            return AM_E_ARG;
        }
    }
    for (int k = 0; k < s.n_nodes; k++) {
        int c0 = s.node_child0[k], nc = s.node_nchild[k];
        if (c0 < 0) continue;   // a leaf
        if (nc < 1 || c0 <= k || c0 > s.n_nodes - nc) {
            err = "sphere-tree node " + std::to_string(k) + ": its children must follow it inside the node array";
            return AM_E_ARG;
        }
    }
    return AM_OK;
}

int32_t am_set_scene(void* ctx, const am_scene* s) {
    if (!ctx || !s) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (check_scene(*s, c->err)) return AM_E_ARG;
    return c->setScene(*s);
}

int32_t am_set_batch(void* ctx, const am_scene* scenes, int32_t n) {
    if (!ctx || !scenes || n <= 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (c->P.enable_merging) { c->err = "batched scenes need enable_merging = 0"; return AM_E_ARG; }
    for (int s = 0; s < n; s++)
        if (check_scene(scenes[s], c->err)) return AM_E_ARG;
    return c->setBatch(scenes, n);
}

int32_t am_set_batch_options(void* ctx, int32_t threads, double residual_target, int32_t check_every) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (threads != 0 && (threads < 32 || threads > 512 || threads % 32)) { c->err = "threads"; return AM_E_ARG; }
    c->batchThreads = threads;
    c->batchThreadsUser = threads;
    c->batchTol = residual_target;
    c->batchCheck = check_every < 0 ? 0 : check_every;
    return AM_OK;
}

int32_t am_get_batch_stats(void* ctx, am_batch_stats* o) {
    if (!ctx || !o) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    o->n_scenes = c->nScenes;
    o->converged = c->batchConverged;
    o->sweeps_max = c->stats.sweeps;
    o->threads = c->batchThreads;
    o->stage_slots = c->batchCap;
    o->resident_scenes = c->batchResident;
    o->cluster_scenes = c->batchClusterScenes();
    o->cluster_size = c->batchClusterMaxK();
    o->sweeps_sum = c->batchSweepsTotal;
    o->contact_sweeps = c->batchContactSweepsLast;
    o->residual_max = c->stats.residual_rel;
    return AM_OK;
}

int32_t am_set_batch_local_sweeps(void* ctx, int32_t passes) {
    if (!ctx || passes < 1 || passes > 64) return AM_E_ARG;
    ((Ctx*)ctx)->batchInner = passes;
    return AM_OK;
}

int32_t am_set_batch_clusters(void* ctx, int32_t enable) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->clusterAllowed = enable != 0;
    c->clusterEnabled = c->clusterAllowed && c->clusterUsable;   // usable: checked when the batch was loaded
    return AM_OK;
}

int32_t am_set_batch_size_classes(void* ctx, int32_t enable) {
    if (!ctx) return AM_E_ARG;
    ((Ctx*)ctx)->batchClasses = enable != 0;
    return AM_OK;
}

int32_t am_set_batch_cluster_stage(void* ctx, int32_t slots) {
    if (!ctx || slots < 0 || (slots && (slots < 64 || slots % 32))) return AM_E_ARG;
    ((Ctx*)ctx)->clusterCapUser = slots;
    return AM_OK;
}

int32_t am_set_batch_stage(void* ctx, int32_t slots) {
    if (!ctx || slots < 0 || (slots && (slots < 64 || slots % 32))) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->batchCapUser = slots;
    c->batchCap = slots;
    return AM_OK;
}

int32_t am_set_batch_relaxation(void* ctx, double relax, int32_t symmetric) {
    if (!ctx || !(relax > 0.0 && relax < 2.0) || symmetric < 0 || symmetric > 1) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->batchRelax = relax;
    c->batchSym = symmetric;
    return AM_OK;
}

int32_t am_set_batch_critical(void* ctx, double frac, int32_t cap) {
    if (!ctx || !(frac >= 0.0 && frac <= 1.0) || cap < 64 || cap % 32) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->batchCriticalFrac = frac;
    c->batchCriticalCap = cap;
    return AM_OK;
}

int32_t am_set_batch_accel(void* ctx, int32_t mode) {
    if (!ctx || mode < 0 || mode > 1) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->batchAccel = mode;
    c->batchThreads = c->batchThreadsUser;   // shared-memory layouts change: tune again
    c->batchCap = c->batchCapUser;
    return AM_OK;
}

int32_t am_set_residual_target(void* ctx, double residual_target, int32_t check_every) {
    if (!ctx || check_every < 0 || !(residual_target >= 0)) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->solveTol = residual_target;
    c->solveCheck = check_every;
    return AM_OK;
}

int32_t am_set_mixed_form(void* ctx, int32_t form, int32_t refine) {
    if (!ctx || form < -1 || form > 2 || refine < 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->mixedForm = form;
    c->mixedRefine = refine;
    return AM_OK;
}

int32_t am_get_mixed_form(void* ctx, int32_t* form) {
    if (!ctx || !form) return AM_E_ARG;
    *form = ((Ctx*)ctx)->mixedLastForm;
    return AM_OK;
}

int32_t am_get_batch_scene_stats(void* ctx, int32_t* sweeps, float* residual, int32_t* fell_back, int32_t* colours) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->nScenes || !c->bSweeps) return AM_E_STATE;
    int n = c->nScenes;
    if (sweeps) cudaMemcpyAsync(sweeps, c->bSweeps, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream);
    if (residual) cudaMemcpyAsync(residual, c->bRes, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
    if (fell_back) cudaMemcpyAsync(fell_back, c->bFall, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream);
    if (colours) return c->batchColours(colours);
    return c->syncErr();
}

int32_t am_get_batch_scene_chain(void* ctx, int32_t* chain) {
    if (!ctx || !chain) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->nScenes) return AM_E_STATE;
    return c->batchChain(chain);
}

int32_t am_get_batch_scene_ctas(void* ctx, int32_t* ctas) {
    if (!ctx || !ctas) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->nScenes) return AM_E_STATE;
    c->batchSceneCtas(ctas);
    return AM_OK;
}

int32_t am_get_batch_scene_times(void* ctx, int64_t* start_ns, int64_t* end_ns, int32_t* sm) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->nScenes || !c->bTrace) return AM_E_STATE;
    int n = c->nScenes;
    std::vector<long long> tr(3 * (size_t)n);
    cudaMemcpyAsync(tr.data(), c->bTrace, sizeof(long long) * tr.size(), cudaMemcpyDeviceToHost, c->stream);
    int r = c->syncErr();
    if (r) return r;
    long long t0 = 0;
    bool any = false;
    for (int s = 0; s < n; s++)
        if (tr[3 * s] > 0 && (!any || tr[3 * s] < t0)) { t0 = tr[3 * s]; any = true; }
    for (int s = 0; s < n; s++) {
        if (start_ns) start_ns[s] = tr[3 * s] > 0 ? tr[3 * s] - t0 : 0;
        if (end_ns) end_ns[s] = tr[3 * s] > 0 ? tr[3 * s + 1] - t0 : 0;
        if (sm) sm[s] = (int32_t)tr[3 * s + 2];
    }
    return AM_OK;
}

int32_t am_learned_collect(void* ctx, int32_t enable, int32_t capacity) {
    if (!ctx || capacity < 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->learnedCollect(enable, capacity);
}

int32_t am_learned_train(void* ctx, int32_t epochs, int32_t batch, double lr, int32_t normalise, double* last_loss) {
    if (!ctx || epochs < 0 || batch <= 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    float l = 0;
    int r = c->learnedTrain(epochs, batch, (float)lr, &l, normalise);
    if (last_loss) *last_loss = l;
    return r;
}

int32_t am_learned_use(void* ctx, int32_t mode) {
    if (!ctx || mode < 0 || mode > 2) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    int r = c->learnedInit();
    if (r) return r;
    if (mode) {
        if ((r = c->learnedPackInference())) return r;
        c->lReady = true;
    }
    c->lUse = mode;
    return AM_OK;
}

int32_t am_learned_scope(void* ctx, int32_t scope) {
    if (!ctx || scope < 0 || scope > 1) return AM_E_ARG;
    ((Ctx*)ctx)->lScope = scope;
    return AM_OK;
}

int32_t am_learned_weights(void* ctx, float* get, const float* set, float* norm_get, const float* norm_set) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->learnedWeights(get, set, norm_get, norm_set);
}

int32_t am_learned_info(void* ctx, int32_t* n_params, int32_t* n_samples, int32_t* fallback_scenes) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (n_params) *n_params = am::learned_num_params();
    if (n_samples) *n_samples = c->lDn;
    if (fallback_scenes) *fallback_scenes = c->lFallbackScenes;
    return AM_OK;
}

int32_t am_learned_grad(void* ctx, const float* X, const float* Y, int32_t n, float* grad, float* loss) {
    if (!ctx || !X || !Y || n <= 0 || !grad || !loss) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->learnedGrad(X, Y, n, grad, loss);
}

int32_t am_learned_infer(void* ctx, const float* X, int32_t n, float* out, int32_t tensor_cores) {
    if (!ctx || !X || n <= 0 || !out) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->learnedInfer(X, n, out, tensor_cores);
}

int32_t am_learned_infer_noalloc(void* ctx, const float* X, int32_t n, float* out, int32_t tensor_cores) {
    if (!ctx || !X || n <= 0 || !out) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->learnedInferNoAlloc(X, n, out, tensor_cores);
}

int32_t am_step(void* ctx, double dt) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) { c->err = "no scene loaded"; return AM_E_STATE; }
    if (c->nScenes > 0 && c->P.enable_merging) { c->err = "batched scenes need enable_merging = 0"; return AM_E_ARG; }
    return c->step(dt);
}

int32_t am_collide(void* ctx, double dt) {
    (void)dt;
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) { c->err = "no scene loaded"; return AM_E_STATE; }
    c->totalSteps++;
    int r = c->beginStep(0);
    if (!r) r = c->collisionDetection();
    if (!r) r = c->syncErr();
    return r;
}

int32_t am_warm_start(void* ctx) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    int r = c->warmStart();
    return r ? r : c->syncErr();
}

int32_t am_solve(void* ctx, double dt, am_solve_stats* st) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    int r = c->solveLCP(dt, c->P.warm_start != 0);
    if (!r) r = c->readCounts();
    if (!r) c->foldTiming();
    if (!r) r = c->collectStats();
    if (!r && st) *st = c->stats;
    return r;
}

int32_t am_integrate(void* ctx, double dt) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    int r = c->finishStep(dt);
    return r ? r : c->syncErr();
}

int32_t am_get_bodies(void* ctx, am_body_state* out) {
    if (!ctx || !out) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->getBodies(out);
}

int Ctx::setKinematic(int body, const double* axis, double amp, double freq, double dt) {
    if (nScenes > 0) { err = "prescribed motion is for single scenes"; return AM_E_STATE; }
    if (body < 0 || body >= nScene || !axis || !(amp >= 0) || !(freq >= 0) || !(dt > 0) || !std::isfinite(amp) ||
        !std::isfinite(freq) || !std::isfinite(dt)) { err = "bad kinematic body"; return AM_E_ARG; }
    if (!(host.flags[body] & F_PINNED)) { err = "a kinematic body must be pinned"; return AM_E_ARG; }
    if (host.parent[body] >= 0) { err = "a kinematic body cannot be inside a collection"; return AM_E_STATE; }
    for (size_t i = 0; i < kin.size(); i++)
        if (kin[i].body == body) { kin.erase(kin.begin() + i); break; }
    if (amp == 0) return AM_OK;
    if (P.enable_sleeping) { err = "kinematic bodies need sleeping off"; return AM_E_STATE; }
    if ((int)kin.size() >= MAXKIN) { err = "too many kinematic bodies"; return AM_E_CAPACITY; }
    Kinematic q;
    q.body = body;
    if (cudaMemcpyAsync(q.x0, B.x + 3 * body, sizeof(double) * 3, cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        return AM_E_CUDA;
    int r = syncErr();
    if (r) return r;
    for (int k = 0; k < 3; k++) q.axis[k] = axis[k];
    q.amp = amp;
    q.omega = 2.0 * 3.141592653589793 * freq;
    q.dt = dt;
    kin.push_back(q);
    kinSteps = 0;
    return AM_OK;
}

int32_t am_set_kinematic(void* ctx, int32_t body, const double* axis, double amplitude, double frequency_hz,
                         double dt) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->setKinematic(body, axis, amplitude, frequency_hz, dt);
}

int32_t am_put_bodies(void* ctx, const am_body_state* in) {
    if (!ctx || !in) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->putBodies(in);
}

int32_t am_num_contacts(void* ctx, int32_t* n) {
    if (!ctx || !n) return AM_E_ARG;
    *n = ((Ctx*)ctx)->nContacts;
    return AM_OK;
}

int32_t am_get_contacts(void* ctx, am_contacts* out, int32_t capacity, int32_t* n) {
    if (!ctx || !out || !n) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->getContacts(out, capacity, n);
}

int32_t am_set_phase_timing(void* ctx, int32_t enable) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    c->phaseOn = enable != 0;
    for (double& v : c->phase) v = 0.;
    return AM_OK;
}

int32_t am_get_phase_times(void* ctx, double* seconds) {
    if (!ctx || !seconds) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    for (int k = 0; k < AM_NUM_PHASES; k++) seconds[k] = c->phase[k];
    return AM_OK;
}

int32_t am_get_perf(void* ctx, am_perf* out) {
    if (!ctx || !out) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    *out = c->perf;
    out->launches = am::g_launches;
    out->merge_events = c->mergeEvents;
    out->unmerge_events = c->unmergeEvents;
    return AM_OK;
}

int32_t am_get_topology(void* ctx, int32_t* items, int32_t* item_off, int32_t cap_items, int32_t* n_top,
                        int32_t* n_items) {
    if (!ctx || !n_top || !n_items) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->stream) return AM_E_STATE;
    return c->getTopology(items, item_off, cap_items, n_top, n_items);
}

int32_t am_reset_perf(void* ctx) {
    if (!ctx) return AM_E_ARG;
    std::memset(&((Ctx*)ctx)->perf, 0, sizeof(am_perf));
    for (double& v : ((Ctx*)ctx)->phaseDevMs) v = 0.0;
    return AM_OK;
}

int32_t am_check_barrier_timeout(void* ctx, int32_t spin_log2, int32_t* status) {
    if (!ctx || !status || spin_log2 < 1 || spin_log2 > 24) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    if (!c->dc || !c->stream) return AM_E_STATE;
    launch_barrier_timeout_check(c->dc, spin_log2, c->stream);
    int e = 0;
    cudaMemcpyAsync(&e, &c->dc->error, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    const int zero = 0;
    cudaMemcpyAsync(&c->dc->error, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return AM_E_CUDA;
    *status = e;
    return AM_OK;
}

static int merging_ctx(Ctx* c) {
    if (!c->stream || !c->host.cap) { c->err = "no scene loaded"; return AM_E_STATE; }
    if (c->nScenes > 0 || !c->host.anyMerging()) {
        c->err = "phase calls of the merging step need a single scene with merging on";
        return AM_E_STATE;
    }
    return AM_OK;
}

int32_t am_step_phase(void* ctx, int32_t phase, double dt) {
    if (!ctx) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    int r = merging_ctx(c);
    if (r) return r;
    if (phase < AM_MPHASE_COLLIDE || phase > AM_MPHASE_FINISH) { c->err = "unknown step phase"; return AM_E_ARG; }
    if (phase == AM_MPHASE_COLLIDE) {
        c->totalSteps++;
        for (double& v : c->phase) v = 0.;
    }
    r = c->mergingPhase(phase, dt);
    return r ? r : c->syncErr();
}

int32_t am_single_sweep_order(void* ctx, int32_t* refs, int32_t capacity, int32_t* n) {
    if (!ctx || !n || capacity < 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    int r = merging_ctx(c);
    if (r) return r;
    std::vector<int> v;
    if (c->P.update_contacts_in_collections && c->anyCollection() && (r = c->singleSweepOrder(v))) return r;
    *n = (int32_t)v.size();
    if (capacity < (int32_t)v.size()) return AM_E_CAPACITY;
    if (!v.empty() && !refs) return AM_E_ARG;
    for (size_t i = 0; i < v.size(); i++) refs[i] = v[i];
    return AM_OK;
}

int32_t am_single_sweep(void* ctx, const int32_t* refs, int32_t n, double dt) {
    if (!ctx || n < 0 || (n > 0 && !refs)) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    int r = merging_ctx(c);
    if (r) return r;
    std::vector<int> v(refs, refs + n);
    return c->singleSweepRefs(v, dt);
}

int32_t am_merge_tests(void* ctx, am_bpc_tests* out, int32_t capacity, int32_t* n) {
    if (!ctx || !n || capacity < 0) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    std::vector<int> a, b, k, res;
    std::vector<double> m;
    int r = c->mergeTests(a, b, k, res, m);
    if (r) return r;
    *n = (int32_t)a.size();
    if (capacity < (int32_t)a.size()) return AM_E_CAPACITY;
    if (!out) return a.empty() ? AM_OK : AM_E_ARG;
    for (size_t i = 0; i < a.size(); i++) {
        if (out->body1) out->body1[i] = a[i];
        if (out->body2) out->body2[i] = b[i];
        if (out->kind) out->kind[i] = k[i];
        if (out->result) out->result[i] = res[i];
        if (out->metric) out->metric[i] = m[i];
    }
    return AM_OK;
}

int32_t am_get_state(void* ctx, void* buf, int64_t capacity, int64_t* size) {
    if (!ctx || !size || capacity < 0 || (capacity > 0 && !buf)) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    std::vector<uint8_t> blob;
    int r = c->getState(blob);
    if (r) return r;
    *size = (int64_t)blob.size();
    if (capacity < (int64_t)blob.size()) return AM_E_CAPACITY;
    std::memcpy(buf, blob.data(), blob.size());
    return AM_OK;
}

int32_t am_put_state(void* ctx, const void* buf, int64_t size) {
    if (!ctx || !buf || size <= 0) return AM_E_ARG;
    return ((Ctx*)ctx)->putState((const uint8_t*)buf, (size_t)size);
}

int32_t am_get_step_phases(void* ctx, double* ms) {
    if (!ctx || !ms) return AM_E_ARG;
    Ctx* c = (Ctx*)ctx;
    for (int k = 0; k < AM_STEP_PHASES; k++) ms[k] = c->phaseDevMs[k];
    return AM_OK;
}

int32_t am_get_stream(void* ctx, void** stream) {
    if (!ctx || !stream) return AM_E_ARG;
    *stream = (void*)((Ctx*)ctx)->stream;
    return AM_OK;
}

int32_t am_get_stats(void* ctx, am_solve_stats* out) {
    if (!ctx || !out) return AM_E_ARG;
    *out = ((Ctx*)ctx)->stats;
    return AM_OK;
}

}  // extern "C"
