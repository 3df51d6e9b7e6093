// capi.cpp -- TEST INFRASTRUCTURE ONLY: C entry points of the oracle, loaded
// by tests/ (ctypes) and by bench.py's CPU-baseline leg.
#include <cstring>

#include "oracle.hpp"

using namespace orc;

extern "C" {

void* or_create(const am_params* p, const am_scene* s) {
    World* w = new World();
    w->init(*p, *s);
    if (w->badSubs) { delete w; return nullptr; }   // a composite sub-body it cannot place
    return w;
}

void or_destroy(void* h) { delete (World*)h; }

void or_set_params(void* h, const am_params* p) { ((World*)h)->P = *p; }

void or_set_residual_target(void* h, double target, int check) {
    ((World*)h)->resTarget = target;
    ((World*)h)->resCheck = check;
}

void or_step(void* h, double dt) { ((World*)h)->step(dt); }

void or_run(void* h, double dt, int n) {
    World* w = (World*)h;
    for (int i = 0; i < n; i++) w->step(dt);
}

/* Phase entry points, in RigidBodySystem.advanceTime order (no collections). */
void or_begin_step(void* h) {
    World* w = (World*)h;
    w->applyKinematic();
    w->totalSteps++;
    w->clearBodies();
    w->applyExternalForces();
}
void or_collide(void* h) {
    World* w = (World*)h;
    w->updateContactsMap();
    w->collisionDetection();
    w->updateBodyPairContacts();
}
void or_warm_start(void* h) { ((World*)h)->warmStart(); }
void or_solve(void* h, double dt) {
    World* w = (World*)h;
    if (w->P.warm_start) w->redoWarmStart();
    else for (Contact* c : w->contacts) { c->l0 = c->l1 = c->l2 = 0; }
    w->solveLCP(dt);
}

int or_num_contacts(void* h) { return (int)((World*)h)->contacts.size(); }

static void put3(double* d, const V3& v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

void or_get_contacts(void* h, am_contacts* o) {
    World* w = (World*)h;
    for (size_t i = 0; i < w->contacts.size(); i++) {
        const Contact* c = w->contacts[i];
        if (o->body1) o->body1[i] = c->body1->id;
        if (o->body2) o->body2[i] = c->body2->id;
        if (o->bv1) o->bv1[i] = c->bv1;
        if (o->bv2) o->bv2[i] = c->bv2;
        if (o->info) o->info[i] = c->info;
        if (o->frame) {
            put3(o->frame + 12 * i, c->cB1); put3(o->frame + 12 * i + 3, c->nB1);
            put3(o->frame + 12 * i + 6, c->t1B1); put3(o->frame + 12 * i + 9, c->t2B1);
        }
        if (o->jac) {
            const V3* r[12] = {&c->jna_v, &c->jna_w, &c->jnb_v, &c->jnb_w, &c->jt1a_v, &c->jt1a_w,
                               &c->jt1b_v, &c->jt1b_w, &c->jt2a_v, &c->jt2a_w, &c->jt2b_v, &c->jt2b_w};
            for (int k = 0; k < 12; k++) put3(o->jac + 36 * i + 3 * k, *r[k]);
        }
        if (o->violation) { o->violation[2 * i] = c->cv; o->violation[2 * i + 1] = c->prevCv; }
        if (o->lambda) { o->lambda[3 * i] = c->l0; o->lambda[3 * i + 1] = c->l1; o->lambda[3 * i + 2] = c->l2; }
        if (o->bD) {
            o->bD[6 * i] = c->bn; o->bD[6 * i + 1] = c->bt1; o->bD[6 * i + 2] = c->bt2;
            o->bD[6 * i + 3] = c->D00; o->bD[6 * i + 4] = c->D11; o->bD[6 * i + 5] = c->D22;
        }
        if (o->state) o->state[i] = c->state;
        if (o->fresh) o->fresh[i] = c->fresh ? 1 : 0;
    }
}

/* Scene bodies only (ids 0..n_scene-1). */
void or_get_bodies(void* h, am_body_state* o) {
    World* w = (World*)h;
    for (int i = 0; i < w->nScene; i++) {
        const Body& b = w->store[i];
        if (o->x) put3(o->x + 3 * i, b.x);
        if (o->R) { const double* p = &b.theta.m00; for (int k = 0; k < 9; k++) o->R[9 * i + k] = p[k]; }
        if (o->v) put3(o->v + 3 * i, b.v);
        if (o->omega) put3(o->omega + 3 * i, b.omega);
        if (o->sleeping) o->sleeping[i] = b.sleeping ? 1 : 0;
        if (o->parent) o->parent[i] = b.parent ? b.parent->id : -1;
    }
}

/* counters: [0]=PGS sweeps of the last full solve, [1]=merge events,
   [2]=unmerge events, [3]=top-level bodies, [4]=body-pair contacts,
   [5]=collections; change = last max |delta lambda|. */
void or_get_counters(void* h, int64_t* out, double* change) {
    World* w = (World*)h;
    int ncol = 0;
    for (Body* b : w->bodies) if (b->isCollection) ncol++;
    out[0] = w->stats.sweeps; out[1] = w->mergeEvents; out[2] = w->unmergeEvents;
    out[3] = (int64_t)w->bodies.size(); out[4] = (int64_t)w->bodyPairContacts.size(); out[5] = ncol;
    if (change) *change = w->stats.last_change;
}

/* Top-level list with collection members: a body is [id], a collection is
   [-1, member ids in order]; returns the number of items. */
int or_topology(void* h, int32_t* items, int32_t* off, int cap, int32_t* ntop) {
    World* w = (World*)h;
    int k = 0, t = 0;
    for (Body* b : w->bodies) {
        if (off) off[t] = k;
        if (b->isCollection) {
            if (items && k < cap) items[k] = -1;
            k++;
            for (Body* s : b->bodies) { if (items && k < cap) items[k] = s->id; k++; }
        } else {
            if (items && k < cap) items[k] = b->id;
            k++;
        }
        t++;
    }
    if (off) off[t] = k;
    *ntop = t;
    return k;
}

/* Top-level body list (RigidBodySystem.bodies) as ids. */
int or_top_ids(void* h, int32_t* out, int cap) {
    World* w = (World*)h;
    int n = (int)w->bodies.size();
    for (int i = 0; i < n && i < cap; i++) out[i] = w->bodies[i]->id;
    return n;
}

int or_set_kinematic(void* h, int body, const double* axis, double amp, double freq, double dt) {
    World* w = (World*)h;
    if (body < 0 || body >= w->nScene) return -1;
    Body* b = &w->store[body];   // scene bodies by id (the top-level list changes with merges)
    if (!b->pinned || b->parent) return -1;
    for (size_t i = 0; i < w->kin.size(); i++)
        if (w->kin[i].body == b) { w->kin.erase(w->kin.begin() + i); break; }
    if (amp == 0) return 0;
    if (w->P.enable_sleeping) return -1;
    World::Kinematic q;
    q.body = b;
    q.x0[0] = q.body->x.x; q.x0[1] = q.body->x.y; q.x0[2] = q.body->x.z;
    for (int k = 0; k < 3; k++) q.axis[k] = axis[k];
    q.amp = amp;
    q.omega = 2.0 * 3.141592653589793 * freq;
    q.dt = dt;
    w->kin.push_back(q);
    w->kinSteps = 0;
    return 0;
}
}  // extern "C"

/* The merge and unmerge tests on the current state, in the reference's
 * iteration order (BodyPairContact.checkMergeCondition, BodyPairContact.java:
 * 151-177, over CollisionProcessor.bodyPairContacts as Merging.merge walks it,
 * Merging.java:80-82; then the unmerge selection of Merging.unmerge,
 * Merging.java:222-240, per awake collection).  kind 0: merge test of a pair
 * in the collision list, kind 1: unmerge test of a pair inside a collection.
 * metric: the newest entry of the pair's motion-metric history (0 if empty).
 * Returns the number of entries (written up to cap). */
extern "C" int or_merge_tests(void* h, int32_t* body1, int32_t* body2, int32_t* kind, int32_t* result,
                              double* metric, int cap) {
    World* w = (World*)h;
    int n = 0;
    auto put = [&](BPC* p, int k, bool r) {
        if (n < cap) {
            body1[n] = p->body1->id;
            body2[n] = p->body2->id;
            kind[n] = k;
            result[n] = r ? 1 : 0;
            metric[n] = p->motionMetricHist.empty() ? 0.0 : p->motionMetricHist.back();
        }
        n++;
    };
    for (BPC* p : w->bodyPairContacts.v) {
        if (p->inCollection) continue;
        put(p, 0, w->mergeTest(p));
    }
    for (Body* b : w->bodies) {
        if (b->sleeping || !b->isCollection) continue;
        for (BPC* p : b->bpcs.v) {
            if (!p->inCollection) continue;
            put(p, 1, w->unmergeTest(p));
        }
    }
    return n;
}
