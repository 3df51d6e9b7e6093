/*
 * am.h -- C ABI of the GB300 contact hot path (collision, contact setup,
 * warm start, projected Gauss-Seidel with box friction, single sweep inside
 * merged collections, integration).
 *
 * Plain C types only; every call returns an int32 status (AM_OK = 0, negative
 * on error) and never aborts.  Host arrays passed in are borrowed for the
 * duration of the call.  One am_ctx owns its device buffers and one CUDA
 * stream; calls on one context are serialised by the caller (the reference is
 * single threaded).
 *
 * Each entry point names the reference method it replaces (paths are relative
 * to the reference project root, EulalieCoevoet/AdaptiveMerging).
 */
#ifndef AM_H
#define AM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define AM_OK            0
#define AM_E_ARG        (-1)  /* bad argument or unsupported scene feature   */
#define AM_E_CAPACITY   (-2)  /* output buffer too small; *n holds the need  */
#define AM_E_NONFINITE  (-3)  /* a multiplier or velocity became NaN/Inf      */
#define AM_E_TIMEOUT    (-4)  /* a bounded device wait gave up               */
#define AM_E_CUDA       (-5)  /* CUDA runtime error (see am_last_error)      */
#define AM_E_STATE      (-6)  /* call order violated (e.g. no scene loaded)  */

/* ---- body geometry types (RigidBodyGeom* / PlaneRigidBody) ------------- */
#define AM_BOX     0   /* RigidBodyGeomBox: shape = (sx, sy, sz, 0)          */
#define AM_SPHERE  1   /* RigidBodyGeomSphere: shape = (r, 0, 0, 0); 1-node tree */
#define AM_PLANE   2   /* PlaneRigidBody: x = point p, shape = (nx, ny, nz, 0) */
#define AM_TREE    3   /* sphere-tree body (mesh / clump), shape unused      */
#define AM_COMPOSITE 4 /* RigidBodyGeomComposite: geometry from am_scene's sub-bodies;
                          no device path yet, am_set_scene refuses it (AM_E_ARG) */

/* ---- contact state (Contact.ContactState) ------------------------------- */
#define AM_STATE_BROKEN 0
#define AM_STATE_ONEDGE 1
#define AM_STATE_CLEAR  2

/* ---- bounding-volume ids carried in contact keys ----------------------- */
#define AM_BV_NULL (-1)            /* no bounding volume (box colliders)      */
#define AM_BV_PLANE(b) (-2 - (b))  /* PlaneRigidBody.dummyBV of plane body b  */

/* ---- Gauss-Seidel ordering on the device -------------------------------- */
#define AM_ORDER_REFERENCE 0  /* contacts in list order: bit-exact to PGS.java */
#define AM_ORDER_COLOURED  1  /* body-pair groups coloured, colours in parallel */
#define AM_ORDER_MIXED     2  /* AM_ORDER_COLOURED with FP32 sweeps on the correction to an FP64
                                 base point, refined in FP64 (same fixed point, FP64 multipliers) */

/*
 * Solver / system parameters.  Field names and defaults follow the reference
 * parameter objects:
 *   CollisionProcessor.java:1058-1083, Merging.java:30-54, Sleeping.java:25-30,
 *   Contact.java:518, RigidBodySystem.java:544-567.
 * am_params_default() fills the reference defaults.
 */
typedef struct am_params {
    /* CollisionProcessor */
    int32_t iterations;               /* 30   */
    double  tolerance;                /* 1e-5 */
    double  omega;                    /* 1    */
    int32_t iterations_in_collection; /* 1    */
    double  feedback_stiffness;       /* 0.5  */
    int32_t enable_compliance;        /* 1    */
    double  compliance;               /* 1e-3 */
    int32_t restitution_override;     /* 0    */
    double  restitution;              /* 0.5 (used only with override) */
    int32_t friction_override;        /* 0    */
    double  friction;                 /* 0.1 (used only with override) */
    int32_t warm_start;               /* 1    */
    /* RigidBodySystem */
    int32_t use_gravity;              /* 1    */
    double  gravity_amount;           /* 1    */
    double  gravity_angle;            /* 90 (degrees) */
    double  viscous_linear;           /* 1    */
    double  viscous_angular;          /* 1    */
    /* Merging.MergeParameters */
    int32_t enable_merging;           /* 1 */
    int32_t enable_merge_pinned;      /* 1 */
    int32_t enable_merge_cycle;       /* 0 (cycle condition: unsupported, must stay 0) */
    int32_t enable_merge_stable_contact; /* 1 */
    int32_t enable_merge_let_it_breathe; /* 1 */
    int32_t enable_unmerging;         /* 1 */
    int32_t enable_unmerge_friction;  /* 1 */
    int32_t enable_unmerge_normal;    /* 1 */
    int32_t enable_unmerge_relative_motion; /* 1 */
    int32_t update_contacts_in_collections; /* 1 */
    int32_t organize_contacts;        /* 1 */
    int32_t metric_position_level;    /* 0 (must stay 0) */
    int32_t step_accum_merging;       /* 3 */
    int32_t step_accum_unmerging;     /* 3 */
    int32_t steps_between_merge_events; /* 10 */
    double  threshold_merge;          /* 1e-2 */
    double  threshold_unmerge;        /* 2e-2 */
    double  threshold_breath;         /* 1e-5 */
    /* Sleeping.SleepParameters */
    int32_t enable_sleeping;          /* 1 */
    int32_t sleep_step_accum;         /* 10 */
    double  sleep_threshold;          /* 1e-5 */
    /* Contact */
    double  sliding_threshold;        /* 0.01 */
    /* device solver ordering (no reference counterpart) */
    int32_t solver_order;             /* AM_ORDER_REFERENCE */
} am_params;

/*
 * Scene description (structure of arrays, body index = stable body id, which
 * replaces Java object identity in contact keys).  Mass properties follow
 * XMLParser.java:360-447: box inertia m/12 (sy^2+sz^2, ...), sphere 2/5 m r^2.
 * Pinned bodies: mass 0 and zero inertia.  Rotations are row-major
 * (m00 m01 m02 m10 ...).
 */
typedef struct am_scene {
    int32_t        n_bodies;
    const int32_t* type;        /* [n] AM_BOX / AM_SPHERE / AM_PLANE / AM_TREE / AM_COMPOSITE */
    const int32_t* pinned;      /* [n] */
    const double*  x;           /* [3n] centre of mass (plane: point p)        */
    const double*  R;           /* [9n] orientation (theta)                     */
    const double*  v;           /* [3n] */
    const double*  omega;       /* [3n] */
    const double*  mass;        /* [n]  massLinear                              */
    const double*  inertia;     /* [9n] massAngular0 (rest pose)                */
    const double*  friction;    /* [n]  default 0.8                             */
    const double*  restitution; /* [n]  default 0                               */
    const double*  shape;       /* [4n] see AM_BOX ... AM_TREE                  */
    /* sphere trees (BVNode / BVSphere); spheres own a single leaf node */
    int32_t        n_nodes;
    const int32_t* body_root;   /* [n] root node index or -1                    */
    const double*  node_c;      /* [3*n_nodes] centre in body frame (cB)        */
    const double*  node_r;      /* [n_nodes]                                    */
    const int32_t* node_child0; /* [n_nodes] first child index or -1 (leaf)     */
    const int32_t* node_nchild; /* [n_nodes] children are contiguous            */
    /* optional, may be NULL: boundingBoxB of AM_TREE bodies as (ll, ur) in
     * body coordinates, [6n].  The motion metric of merging and sleeping
     * samples the velocity at its 8 corners (MotionMetricProcessor.java:
     * 39-73).  A mesh body's box is its mesh's (XMLParser.java:474-493);
     * NULL, non-finite entries and other body types take the box of the
     * geometry (AM_TREE: the box of its leaf spheres). */
    const double*  bbox;
    /* composite bodies (RigidBodyGeomComposite, XMLParser.java:180-352): the
     * sub-bodies of the AM_COMPOSITE bodies, in each composite's list order,
     * with stable ids (their index here) in place of Java object identity.
     * A sub-body is a box (sub_shape = size) or a sphere (sub_shape[0] = r)
     * with its pose in the composite's frame (transformB2C: sub_R, sub_t).
     * n_subs = 0 without composites. */
    int32_t        n_subs;
    const int32_t* sub_parent;  /* [n_subs] index of the composite body       */
    const int32_t* sub_type;    /* [n_subs] AM_BOX / AM_SPHERE                 */
    const double*  sub_shape;   /* [4*n_subs]                                  */
    const double*  sub_R;       /* [9*n_subs] rotation in the composite frame  */
    const double*  sub_t;       /* [3*n_subs] position in the composite frame  */
} am_scene;

/* Per-body state read back after a step. */
typedef struct am_body_state {
    double*  x;       /* [3n] */
    double*  R;       /* [9n] */
    double*  v;       /* [3n] */
    double*  omega;   /* [3n] */
    int32_t* sleeping;/* [n]  */
    int32_t* parent;  /* [n]  collection id or -1 */
} am_body_state;

/*
 * Contacts read back in list order.  Frame quantities are stored as the
 * reference stores them (Contact.java:199-224): contact point, normal and
 * tangents in body-1 coordinates; Jacobian rows in world coordinates.
 */
typedef struct am_contacts {
    int32_t* body1;      /* [c] */
    int32_t* body2;      /* [c] */
    int32_t* bv1;        /* [c] node id / AM_BV_NULL / AM_BV_PLANE(b) */
    int32_t* bv2;        /* [c] */
    int32_t* info;       /* [c] */
    double*  frame;      /* [12c] contactB1, normalB1, tangent1B1, tangent2B1 */
    double*  jac;        /* [36c] jna, jnb, jt1a, jt1b, jt2a, jt2b (v then w) */
    double*  violation;  /* [2c] constraintViolation, prevConstraintViolation */
    double*  lambda;     /* [3c] lambda0..2 */
    double*  bD;         /* [6c] bn, bt1, bt2, D00, D11, D22 */
    int32_t* state;      /* [c] AM_STATE_* */
    int32_t* fresh;      /* [c] newThisTimeStep */
} am_contacts;

typedef struct am_solve_stats {
    int32_t n_contacts;      /* contacts in the full solve                       */
    int32_t sweeps;          /* PGS iterations run (early exit on tolerance)     */
    double  last_change;     /* max |delta lambda| of the last sweep             */
    double  residual_abs;    /* natural-map LCP residual, inf-norm               */
    double  residual_rel;    /* residual_abs / max(1, |lambda|_inf)              */
} am_solve_stats;

/* Performance counters of one context (no reference counterpart; used by the
 * benchmark to compute the roofline of the PGS sweep kernel). */
typedef struct am_perf {
    int64_t launches;        /* kernels launched by libam since it was loaded   */
    int64_t pgs_launches;    /* full-solve PGS sweep launches of this context  */
    double  pgs_ms;          /* their summed device time (CUDA events on the context stream) */
    int64_t contact_sweeps;  /* sum of contacts x sweeps over those launches    */
    int64_t steps;           /* am_step calls                                   */
    int64_t merge_events;    /* body pairs merged since the scene was loaded    */
    int64_t unmerge_events;  /* collections split since the scene was loaded    */
} am_perf;

/* ---- lifecycle ---------------------------------------------------------- */
void        am_params_default(am_params* p);
/* new context on the current CUDA device */
int32_t     am_create(const am_params* p, void** ctx);
int32_t     am_destroy(void* ctx);
const char* am_last_error(void* ctx);
int32_t     am_set_params(void* ctx, const am_params* p);

/* Load a scene (replaces RigidBodySystem.bodies + reset(), RigidBodySystem.java:78,390-426). */
int32_t am_set_scene(void* ctx, const am_scene* scene);

/* One full step: RigidBodySystem.advanceTime(dt), RigidBodySystem.java:102-185. */
int32_t am_step(void* ctx, double dt);

/* CollisionProcessor.updateContactsMap + collisionDetection (CollisionProcessor.java:443-448, 91-102). */
int32_t am_collide(void* ctx, double dt);
/* CollisionProcessor.warmStart(false) (CollisionProcessor.java:481-640). */
int32_t am_warm_start(void* ctx);
/* CollisionProcessor.solveLCP(dt,false) -> PGS.solve (CollisionProcessor.java:108-137, PGS.java:73-194). */
int32_t am_solve(void* ctx, double dt, am_solve_stats* stats);
/* RigidBody.advanceVelocities + advancePositions for all bodies (RigidBody.java:409-441). */
int32_t am_integrate(void* ctx, double dt);

/*
 * The step with merging on, one phase at a time, so a host can keep its own
 * orchestration between them (read am_merge_tests before the merge phase,
 * run the single sweep in its own contact order).  Calling the phases 0..7 in
 * order is am_step.  Phases follow RigidBodySystem.advanceTime
 * (RigidBodySystem.java:102-185); AM_E_STATE on a batched context or with
 * merging off (am_collide / am_warm_start / am_solve / am_integrate cover
 * that step).
 */
enum {
    AM_MPHASE_COLLIDE = 0,      /* forces, updateContactsMap, collisionDetection, updateBodyPairContacts (:110-124); counts the step */
    AM_MPHASE_WARM_START = 1,   /* warmStart(false), sleeping.wake (:126-132) */
    AM_MPHASE_SINGLE_SWEEP = 2, /* updateInCollections (:135) in the reference's contact order */
    AM_MPHASE_UNMERGE = 3,      /* accumulateForUnmerging, merging.unmerge, forces again after an event (:138-147) */
    AM_MPHASE_SOLVE = 4,        /* redoWarmStart, solveLCP, clearBodyPairContacts (:150-157) */
    AM_MPHASE_ADVANCE = 5,      /* advanceBodiesVelocities, accumulateForMerging, advanceBodiesPositions (:160-166) */
    AM_MPHASE_MERGE = 6,        /* merging.merge every steps_between_merge_events steps (:171-173) */
    AM_MPHASE_FINISH = 7        /* sleeping.sleep (:176) and the step's counters */
};
int32_t am_step_phase(void* ctx, int32_t phase, double dt);
/* The contacts the single sweep of this step visits, in the order of
 * CollisionProcessor.getOrganizedContacts (CollisionProcessor.java:337-364,
 * breadth-first layers from the pairs with fresh contacts): refs[i] >= 0 is
 * contact refs[i] of the current list, refs[i] < 0 is the contact inside a
 * collection at slot ~refs[i].  Valid after AM_MPHASE_WARM_START; AM_E_CAPACITY
 * with *n set when capacity is too small. */
int32_t am_single_sweep_order(void* ctx, int32_t* refs, int32_t capacity, int32_t* n);
/* In place of AM_MPHASE_SINGLE_SWEEP: the single sweep of
 * CollisionProcessor.updateInCollections (CollisionProcessor.java:262-302,
 * PGS.java:73-194 with iterations_in_collection passes) over the given
 * contacts in the given order, then the collections' sub-body velocities.
 * AM_E_ARG for a reference out of range. */
int32_t am_single_sweep(void* ctx, const int32_t* refs, int32_t n, double dt);

/*
 * The merge and unmerge predicates on the state at the end of the last step,
 * read only (nothing is merged or split): for a host that keeps its own
 * merging logic and needs the decisions' inputs.  Entries come in the
 * reference's iteration order: first every body-pair contact of the
 * collision list that is not inside a collection, with
 * BodyPairContact.checkMergeCondition (BodyPairContact.java:151-177) in
 * Merging.merge's walk (Merging.java:80-82, kind 0); then every pair inside
 * an awake collection, with Merging.unmerge's selection test
 * (checkContactsState or the relative-motion history, Merging.java:222-240,
 * BodyPairContact.java:255-266, kind 1).  metric is the newest entry of the
 * pair's motion-metric history (0 when empty).  AM_E_CAPACITY with *n set
 * when capacity is too small; AM_E_STATE on a batched context.
 */
typedef struct am_bpc_tests {
    int32_t* body1;   /* [cap] */
    int32_t* body2;   /* [cap] */
    int32_t* kind;    /* [cap] 0 merge test, 1 unmerge test */
    int32_t* result;  /* [cap] 1 when the pair is a candidate */
    double*  metric;  /* [cap] */
} am_bpc_tests;
int32_t am_merge_tests(void* ctx, am_bpc_tests* out, int32_t capacity, int32_t* n);

/*
 * Snapshot and restore between steps.  The reference rebuilds its state from
 * Java objects (RigidBodySystem.reset, RigidBodySystem.java:390-426; the
 * contact pool, ContactPool.java:23-73; body-pair contacts with their
 * motion-metric and contact-state histories, BodyPairContact.java:83-145;
 * collections, RigidCollection.java).  am_get_state writes all of the
 * context's state into one byte blob: bodies (with collections and sleeping
 * histories), the last step's contacts with multipliers and warm-start copies,
 * contacts inside collections, body-pair contacts and their histories, the
 * step counter.  With capacity too small (or 0) it returns AM_E_CAPACITY and
 * the size needed in *size.  am_put_state restores a blob into a context
 * loaded with the same scene (am_set_scene / am_set_batch with the same
 * bodies; AM_E_STATE otherwise, AM_E_ARG for a malformed blob): the steps that
 * follow are bit-identical to those that followed the snapshot.  The blob is
 * for this library build only.
 */
int32_t am_get_state(void* ctx, void* buf, int64_t capacity, int64_t* size);
int32_t am_put_state(void* ctx, const void* buf, int64_t size);

/* Read back. */
int32_t am_get_bodies(void* ctx, am_body_state* out);
/* Write x / R / v / omega of the free scene bodies (a caller that owns the
 * body objects, as the Java RigidBody list does, pushes its state before a
 * step); bodies inside a collection follow their collection and are skipped.
 * Replaces the state the reference keeps in RigidBody.x/theta/v/omega
 * (RigidBody.java:89-96). */
int32_t am_put_bodies(void* ctx, const am_body_state* in);
int32_t am_num_contacts(void* ctx, int32_t* n);
int32_t am_get_contacts(void* ctx, am_contacts* out, int32_t capacity, int32_t* n);
int32_t am_get_stats(void* ctx, am_solve_stats* out);

/*
 * Batched scenes (no reference counterpart: the reference simulates one
 * scene).  n independent scenes are loaded into one context; am_step then
 * advances all of them (collision per scene; in the solve one CTA per scene,
 * launched in size classes, or a thread-block cluster of 2-8 CTAs for a scene
 * too large for one CTA's shared memory).  Body ids in readbacks are global: scene s's body i is at
 * (number of bodies of scenes < s) + i.  Merging must be off.  The batched
 * solve runs in FP32 with delta-v in shared memory and stops each scene when
 * its relative natural-map residual is <= residual_target (checked every
 * check_every sweeps) or after am_params.iterations sweeps.  A scene whose
 * bodies do not fit one CTA's shared memory (about 4000 bodies) is refused
 * with AM_E_CAPACITY.
 */
typedef struct am_batch_stats {
    int32_t n_scenes;
    int32_t converged;       /* scenes that reached the residual target        */
    int32_t sweeps_max;      /* largest sweep count of the last step           */
    int32_t threads;         /* threads per scene CTA (autotuned when 0 given) */
    int32_t stage_slots;     /* contact records per shared-memory staging buffer (autotuned) */
    int32_t resident_scenes; /* scenes whose records stayed in shared memory, last step */
    int32_t cluster_scenes;  /* scenes solved by a thread-block cluster, last step */
    int32_t cluster_size;    /* CTAs in the largest cluster used, last step (0: none) */
    int64_t sweeps_sum;      /* sum of the scenes' sweep counts, last step     */
    int64_t contact_sweeps;  /* sum of contacts x sweeps, last step            */
    double  residual_max;    /* worst scene residual, last step                */
} am_batch_stats;
int32_t am_set_batch(void* ctx, const am_scene* scenes, int32_t n_scenes);
/* threads: 0 = autotune on the first step; residual_target <= 0 disables the test */
int32_t am_set_batch_options(void* ctx, int32_t threads, double residual_target, int32_t check_every);
int32_t am_get_batch_stats(void* ctx, am_batch_stats* out);
/* passes of each sweep over one body pair's contacts (1 = plain PGS; more is
 * block Gauss-Seidel on the pair, same fixed point).  No reference counterpart. */
int32_t am_set_batch_local_sweeps(void* ctx, int32_t passes);
/* 1 (default): scenes too large for one CTA's shared memory are solved by a
 * thread-block cluster of 2-8 CTAs; 0: they stream through one CTA. */
int32_t am_set_batch_clusters(void* ctx, int32_t enable);
/* 1 (default): every scene that fits one CTA's shared memory is solved by one
 * of the size-class launches, whose CTAs are sized for the class (small ones
 * several to an SM); 0: such scenes share the one-CTA launch, whose staging
 * capacity is autotuned.  Results are the same either way.  No reference
 * counterpart. */
int32_t am_set_batch_size_classes(void* ctx, int32_t enable);
/* contact records per shared-memory staging buffer of the one-CTA kernel
 * (a multiple of 32, at least 64; 0 = autotuned) */
int32_t am_set_batch_stage(void* ctx, int32_t slots);
/* contact records each CTA of a cluster holds (a multiple of 32, at least 64;
 * 0 = the largest that fits, at most 2048); takes effect at the next am_set_batch */
int32_t am_set_batch_cluster_stage(void* ctx, int32_t slots);
/* batched sweep variants with the same fixed point (no reference counterpart):
 * over-relaxation factor in (0, 2) applied before the projection (1 = plain
 * PGS), and symmetric = 1 to walk the colours backwards on odd sweeps */
int32_t am_set_batch_relaxation(void* ctx, double relax, int32_t symmetric);
/* 1: every batched sweep is wrapped in a nonsmooth nonlinear conjugate-
 * gradient step (Silcowitz, Niebe and Erleben 2010): with g the sweep's change
 * of the multipliers and beta = |g_k|^2 / |g_k-1|^2, lambda += beta p and
 * p = beta p + g, restarting (p = 0) when beta > 1.  Same fixed point as
 * projected Gauss-Seidel, so the residual stopping rule is unchanged; results
 * stay independent of CTA size, size classes, staging and clusters.  0 (default): plain
 * projected Gauss-Seidel, PGS.java:73-194.  Wraps the reference's sweep; no
 * reference counterpart. */
int32_t am_set_batch_accel(void* ctx, int32_t mode);
/* the split of a large scene over a cluster: a scene whose last solve cost at
 * least frac (0..1) of the batch's costliest one is critical, and each CTA of
 * its cluster holds at most cap records (a multiple of 32, >= 64), so it runs
 * on more CTAs and finishes sooner.  Default 0.75 and 640.  Results do not
 * depend on it.  No reference counterpart. */
int32_t am_set_batch_critical(void* ctx, double frac, int32_t cap);
/* coloured full solve of a single scene (AM_ORDER_COLOURED): stop once the
 * relative natural-map residual is <= residual_target, tested every
 * check_every sweeps (0 disables; the reference's max-change tolerance still
 * applies).  No reference counterpart: PGS.java stops on max |delta lambda| only. */
int32_t am_set_residual_target(void* ctx, double residual_target, int32_t check_every);
/* A pinned body moved by a prescribed oscillation (a shaking platform).  No
 * reference counterpart: the reference's pinned bodies stand still; a moving
 * support enters the contact path only through the body velocity that
 * Contact.computeB reads (Contact.java:290-321), the path a pinned body's zero
 * velocity already takes (RigidBody.java:50).  At the start of the n-th step
 * after this call (n = 0, 1, ...), the body's position is
 *   x0 + axis * (amplitude * sin(w n dt)),  velocity axis * ((amplitude * w) * cos(w n dt)),
 * w = 2 pi frequency_hz, x0 its position at this call; its orientation is
 * unchanged.  The body must be pinned (AM_E_ARG otherwise); amplitude 0 removes
 * it; at most 8 per context (AM_E_CAPACITY); single scenes only (AM_E_STATE
 * for a batch).  Setting any body restarts the count n of every one.  A
 * kinematic body never merges (its pairs fail the merge test, the one
 * addition to BodyPairContact.checkMergeCondition): a collection holding a
 * pinned body stays put, so the motion would stop acting on its contacts.  A
 * body already inside a collection is refused (AM_E_STATE), and so is a
 * kinematic body while sleeping is on, here and in am_set_params: the
 * reference's sleeping treats every pinned body as static (the broad phase
 * skips pinned-sleeping pairs, CollisionProcessor.java:693-694, and contacts
 * with pinned bodies neither keep a body awake nor wake it,
 * Sleeping.java:65-72, 107-121), so a moving support would pass through a body asleep
 * on it.  Loading a new scene or batch clears every kinematic body. */
int32_t am_set_kinematic(void* ctx, int32_t body, const double* axis, double amplitude, double frequency_hz,
                         double dt);
/* AM_ORDER_MIXED: the form of the solve kernel (-1, default: chosen per
 * step from the colours and sizes; 0: a cooperative grid; 1: one block, body
 * data in shared memory; 2: one block, contact records in shared memory too,
 * taken only when they fit) and the FP64 refinement interval in sweeps (0,
 * default: every 100 sweeps, or at every residual check when a residual target
 * is set).  Results do not depend on the form beyond FP32 rounding.  No
 * reference counterpart. */
int32_t am_set_mixed_form(void* ctx, int32_t form, int32_t refine);
/* the form the last AM_ORDER_MIXED solve ran in (-1 before the first) */
int32_t am_get_mixed_form(void* ctx, int32_t* form);
/* per-scene figures of the last step (arrays of n_scenes; NULL skips one):
 * sweeps, relative residual, learned start fell back, colours of the contact groups */
int32_t am_get_batch_scene_stats(void* ctx, int32_t* sweeps, float* residual, int32_t* fell_back, int32_t* colours);
/* per scene, last batched solve: start and end of its sweep kernel CTA (ns,
 * relative to the earliest start) and the SM it ran on (a cluster: its first
 * CTA).  Any pointer may be null.  No reference counterpart. */
int32_t am_get_batch_scene_times(void* ctx, int64_t* start_ns, int64_t* end_ns, int32_t* sm);
/* per scene, last batched solve: CTAs that solved it (1: one CTA, a size
 * class or the streaming launch; 2, 4 or 8: a thread-block cluster).  No
 * reference counterpart. */
int32_t am_get_batch_scene_ctas(void* ctx, int32_t* ctas);
/* per scene, last batched solve: the critical path of one sweep in contacts,
 * the sum over the scene's colours of its longest body-pair group (the
 * contacts of a group update one after another; a colour ends with its
 * longest group).  Sweeps x this x the cycles of one contact update bound the
 * scene's solve time from below.  No reference counterpart. */
int32_t am_get_batch_scene_chain(void* ctx, int32_t* chain);

/*
 * Learned warm start for the batched solve (no reference counterpart).  An
 * MLP 24 -> 64 -> 64 -> 3 (GELU) maps per-contact features to the converged
 * multipliers; it is trained on the device by the library's own forward,
 * backward and Adam kernels from (features, converged multiplier) pairs that
 * the plain solver records, and evaluated with BF16 weights on the tensor
 * cores.  Scenes that miss the residual target from the learned start are
 * solved again from the plain previous-frame warm start.
 */
/* record (features, converged multipliers) of converged scenes during am_step */
int32_t am_learned_collect(void* ctx, int32_t enable, int32_t capacity);
/* mini-batch Adam over the recorded samples; normalise = 1 recomputes feature scaling */
int32_t am_learned_train(void* ctx, int32_t epochs, int32_t batch, double lr, int32_t normalise, double* last_loss);
/* 0: plain warm start; 1: learned start, BF16 tensor-core inference; 2: learned start, FP32 inference */
int32_t am_learned_use(void* ctx, int32_t mode);
/* which contacts are recorded and take the learned start: 0 fresh contacts (default), 1 all contacts */
int32_t am_learned_scope(void* ctx, int32_t scope);
/* get / set the FP32 parameters (n_params floats) and the feature scaling (48 floats); NULL skips */
int32_t am_learned_weights(void* ctx, float* get, const float* set, float* norm_get, const float* norm_set);
/* n_params, recorded samples, scenes that fell back to the plain start in the last step */
int32_t am_learned_info(void* ctx, int32_t* n_params, int32_t* n_samples, int32_t* fallback_scenes);
/* loss and gradient of the current parameters on n samples (X: n x 24, Y: n x 3, row-major) */
int32_t am_learned_grad(void* ctx, const float* X, const float* Y, int32_t n, float* grad, float* loss);
/* network outputs for n feature rows; tensor_cores = 1 uses the BF16 kernel */
int32_t am_learned_infer(void* ctx, const float* X, int32_t n, float* out, int32_t tensor_cores);

/*
 * am_learned_infer without allocation (no counterpart in the reference).
 * Same arguments and results as am_learned_infer, but the rows pass through a
 * fixed device scratch of AM_NOALLOC_MAX_ROWS rows (7.1 MB per device)
 * instead of device temporaries allocated and freed by every call.  It is for
 * hosts that must not allocate inside their step loop: a real-time JNI / FFM
 * thread, where cudaMalloc / cudaFree can stall on device-wide
 * synchronisation, and hosts that reserve the device memory for their own
 * pool up front and leave the library none to take mid-run.
 *   - needs the context's weights set up first (am_learned_use with a
 *     mode > 0, am_learned_weights with weights to set, or
 *     am_learned_train), else AM_E_STATE;
 *   - the context's device (current at am_create) must be the current
 *     device, else AM_E_STATE;
 *   - n > AM_NOALLOC_MAX_ROWS returns AM_E_CAPACITY, n <= 0 AM_E_ARG;
 *   - errors are reported by the status alone (am_last_error is not updated);
 *   - the first call on a device, made with that device current, looks up
 *     the scratch's address; make that first call before any stream capture;
 *   - calls that overlap in time on one device share the scratch and race:
 *     serialise them.
 */
#define AM_NOALLOC_MAX_ROWS 65536
int32_t am_learned_infer_noalloc(void* ctx, const float* X, int32_t n, float* out, int32_t tensor_cores);

/* Top-level body list (RigidBodySystem.bodies, RigidBodySystem.java:31) with
 * collection membership (RigidCollection.bodies, RigidCollection.java:28):
 * entry t spans items[item_off[t] .. item_off[t+1]); a free body is [id], a
 * collection is [-1, member ids in order].  item_off needs n_top + 1 slots. */
int32_t am_get_topology(void* ctx, int32_t* items, int32_t* item_off, int32_t cap_items, int32_t* n_top,
                        int32_t* n_items);

/* Instrumentation (no reference counterpart). */
int32_t am_get_perf(void* ctx, am_perf* out);
int32_t am_reset_perf(void* ctx);

/* Per-phase wall times of the last am_step, in seconds, in the order of the
 * reference's CSV columns (RigidBodySystem.exportDataToFile,
 * RigidBodySystem.java:495-542; measured at RigidBodySystem.java:102-175,
 * CollisionProcessor.java:91-302, Merging.java:73-273).  Off by default: when
 * on, every phase boundary synchronises the context stream, so the phases
 * are wall times of the device work, as the reference's are of its Java
 * work.  Phases that do not run (no merging, no collections) read 0. */
enum {
    AM_PHASE_DETECTION = 0,          /* collisionDetectTime  */
    AM_PHASE_WARMSTART = 1,          /* warmStartTime        */
    AM_PHASE_LCP_SOLVE = 2,          /* collisionSolveTime   */
    AM_PHASE_UPDATE_COLLECTIONS = 3, /* collectionUpdateTime */
    AM_PHASE_CONTACT_ORDERING = 4,   /* contactOrderingTime  */
    AM_PHASE_SINGLE_IT_PGS = 5,      /* singleItPGSTime      */
    AM_PHASE_MERGING = 6,            /* mergingTime          */
    AM_PHASE_MERGING_BUILD = 7,      /* mergingBuildTime     */
    AM_PHASE_UNMERGING = 8,          /* unmergingTime        */
    AM_PHASE_UNMERGING_BUILD = 9,    /* unmergingBuildTime   */
    AM_PHASE_COMPUTE = 10,           /* computeTime          */
    AM_NUM_PHASES = 11
};
int32_t am_set_phase_timing(void* ctx, int32_t enable);
int32_t am_get_phase_times(void* ctx, double* seconds /* [AM_NUM_PHASES] */);
/* Device time of the phases of the batched am_step, in milliseconds summed
 * over the steps since am_reset_perf, measured with CUDA events at the phase
 * boundaries on the context stream: detection, warm start, solve set-up
 * (contact setup, colouring, record packing, launch planning), the sweep
 * launches, integration, statistics.  Boundaries are consecutive, so the
 * phases add up to the device time of the steps, including the time the
 * device waits on the host between phases.  No reference counterpart. */
#define AM_STEP_PHASES 6
int32_t am_get_step_phases(void* ctx, double* ms /* [AM_STEP_PHASES] */);
/* Self-check of the bounded grid barrier of the FP64 sweeps: two blocks wait
 * at a barrier that cannot complete, each giving up after 2^spin_log2 polls
 * (1..24).  *status receives the device status word (AM_E_TIMEOUT when the
 * bound works), which is then cleared; the context stays usable.  No
 * reference counterpart. */
int32_t am_check_barrier_timeout(void* ctx, int32_t spin_log2, int32_t* status);
/* the context's cudaStream_t, for callers that order their own work after a step */
int32_t am_get_stream(void* ctx, void** stream);

#ifdef __cplusplus
}
#endif
#endif /* AM_H */
