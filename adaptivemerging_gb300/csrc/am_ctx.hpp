// am_ctx.hpp -- device data layout and the internal kernel entry points of
// libam.  Not part of the public ABI (include/am.h).
//
// HBM layout (FP64 drop-in):
//   bodies   : per-body records, vectors stored xyz-contiguous (x[3i+k]),
//              matrices row-major 9 doubles (R[9i+k]); a body slot exists for
//              every scene body and every collection the host creates.
//   nodes    : sphere-tree nodes (cB, r, child0, nchild, owner, cW).
//   contacts : structure of arrays with a per-field stride of `cap`
//              (J[k*cap + c] for k = 0..35) so that a warp reading one field
//              of 32 consecutive contacts issues one coalesced 256 B request.
//              Two buffers alternate every step (the previous step's
//              contacts are the warm-start donors, as ContactPool.swapPools
//              keeps them).
//   pairs    : body-pair groups of the current step; contacts of one pair are
//              a contiguous run [poff, poff + pcount) in list order.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/am.h"

namespace am {

// kernels launched by this library since load (read by am_get_perf)
extern long long g_launches;
#define AM_LAUNCHED(n) (::am::g_launches += (n))

enum : int { F_PINNED = 1, F_SLEEPING = 2, F_COLLECTION = 4 };

struct DBodies {
    int n;
    int* type;
    int* flags;
    int* parent;     // collection slot or -1
    int* root;       // sphere-tree root node or -1
    double* x;       // 3
    double* R;       // 9
    double* v;       // 3
    double* w;       // 3
    double* mass;    // massLinear
    double* minv;
    double* jinv;    // 9
    double* jinv0;   // 9
    double* M;       // massAngular 9
    double* M0;      // massAngular0 9
    double* force;   // 3
    double* torque;  // 3
    double* dv;      // 6 (v then w)
    double* size;    // 3 (box)
    double* radius;
    double* friction;
    double* restitution;
    double* plane;   // 4: n, d
    double* pp;      // 3: plane point p
    double* bbB;     // 24
    double* hist;    // sleep metric history (HIST per body, ring)
    int* hist_n;     // number of valid entries
    int* hist_h;     // ring head
    double* B2C;     // 12: R(9) t(3) body-to-collection
    float4* bc;      // broad-phase prefilter: bounding centre and radius in FP32 (w < 0: no prefilter)
};
static const int HIST = 16;

struct DNodes {
    int n;
    double* cB;      // 3
    double* cW;      // 3
    double* r;
    int* child0;
    int* nchild;
    int* body;
};

struct DContacts {
    int cap;
    int *b1, *b2, *bv1, *bv2, *info, *pair, *state, *fresh;
    double* f;       // 12 * cap : contactB1, normalB1, tangent1B1, tangent2B1
    double* J;       // 36 * cap : jna.v jna.w jnb.v jnb.w jt1a.v ... (k*cap + c)
    double* cv;      // constraintViolation
    double* pcv;     // prevConstraintViolation
    double* lam;     // 3 * cap
    double* lamw;    // 3 * cap (warm-start copy)
    double* bD;      // 6 * cap : bn bt1 bt2 D00 D11 D22
    double* Ia;      // 9 * cap : jinv_1 * J_row.w for the three rows (solve body 1)
    double* Ib;      // 9 * cap
    int *sb1, *sb2;  // solve bodies (parent collection when merged, else the body)
};

struct DPairs {
    int cap;
    int *a, *b;      // body slots (sub-bodies for collection pairs)
    int* count;      // contacts of the pair
    int* off;        // first contact
    int* keep;       // pair survives clearBodyPairContacts
    int* perm;       // narrow-phase processing order: pairs grouped by body-type class
};

struct Scratch {
    int cap_int;
    int* tmp;        // scan input scratch
    int* tmp2;       // scan output scratch
    int* block;      // block sums: cap_int / 1024 + 2 first-level sums, then 1024 second-level ones
    int cap_block;
};

// device-side counters and flags (one struct in device memory)
struct DCount {
    int n_cand;      // broad-phase candidate pairs
    int n_pairs;     // narrow-phase pairs (sub-body pairs)
    int n_contacts;  // contacts emitted
    int overflow;    // capacity exceeded (required size in need_*)
    int need_contacts;
    int need_pairs;
    int sweeps;
    int error;       // AM_E_* raised on device
    // max |delta lambda| of a sweep (bits of a non-negative double), slot sweep % 3: a sweep
    // clears the next sweep's slot before its own last barrier, after every reader of
    // that slot's previous use passed the barrier before (with two slots a one-colour
    // sweep could clear a slot that another block had already written)
    unsigned long long maxchg[3];
    int n_colours;
    int bar_count;   // grid-barrier arrivals of the running cooperative sweep (counts up)
    double res_abs;  // residual
    double lam_max;
    int n_prev;      // contacts in the previous buffer
    unsigned long long reschk[2];  // residual-target check of the coloured solve (double bits, by check parity)
    unsigned long long lamchk[2];
    int stage_ovf;   // the staged narrow phase met a pair with more contacts than it keeps
    int spin_log2;   // grid barriers give up after 2^spin_log2 polls (0: 2^24)
};

// ---- kernels / launchers (defined in the .cu files) ----------------------
void launch_begin_step(const DBodies& B, const int* top, int ntop, double gx, double gy, double gz,
                       int mergingReapply, cudaStream_t s);
void launch_bv_update(const DBodies& B, const DNodes& N, cudaStream_t s);
// narrow-phase order: pairs grouped by body-type class (box-plane, sphere-tree
// on plane, box-box, box-tree, tree-tree), so a warp runs one collider; cls
// is 16 ints of device scratch
void launch_pair_order(const DBodies& B, DPairs& P, int n, int* cls, cudaStream_t s);
int launch_broadphase(const DBodies& B, const DNodes& N, const int* top, int ntop, int* candA, int* candB,
                      int candCap, int* rowCount, int* rowOff, Scratch& sc, DCount* dc, cudaStream_t s,
                      const int* topEnd = nullptr, unsigned* masks = nullptr, int mw = 0);
// FP32 bounding centre and radius of the members of collections (DBodies::bc)
void launch_broad_pack_subs(const DBodies& B, const DNodes& N, const int* subIds, int nsub, cudaStream_t s);
void launch_expand_pairs(const DBodies& B, const int* sub_off, const int* sub_ids, const int* candA,
                         const int* candB, int ncand, DPairs& P, Scratch& sc, DCount* dc, cudaStream_t s);
void launch_narrow(const DBodies& B, const DNodes& N, DPairs& P, DContacts& C, Scratch& sc, DCount* dc,
                   bool emit, cudaStream_t s, double* sd = nullptr, int* si = nullptr, int* ovf = nullptr);
int narrow_stage_slots();
void launch_scan(const int* in, int* out, int n, Scratch& sc, int* total, cudaStream_t s);

// solve.cu
struct DHash {
    int cap;         // power of two
    int* slot;       // contact index in the previous buffer or -1
};
void launch_ws_build(const DContacts& prev, int nprev, DHash& H, cudaStream_t s);
void launch_warm_start(const DBodies& B, DContacts& cur, DContacts& prev, const DHash& H, DPairs& P,
                       int npairs, int nprev, cudaStream_t s);
void launch_solve_prep(const DBodies& B, DContacts& C, int nc, double dt, double fb, bool inColl,
                       int restOv, double restVal, int redoWarm, cudaStream_t s);
void colour_groups(const DBodies& B, const DContacts& C, DPairs& P, int npairs, int* colourOf, int* colourCnt,
                   int* colourOff, int* fill, int* groupOrder, int maxC, unsigned long long* bodyMax, int nbodies,
                   DCount* dc, Scratch& sc, cudaStream_t s);
void launch_pgs_fast(const DBodies& B, DContacts& C, DPairs& P, const int* groupOrder, const int* colourOff,
                     int ncol, int nc, int iters, double omega, double comp, double tol, bool early, int fo,
                     double fv, double slide, double* Mj, double* K, int mcap, DCount* dc, int gridBlocks,
                     cudaStream_t s, double resTol = 0.0, int check = 0);
// AM_ORDER_MIXED: the coloured solve's sweeps in FP32 on the correction to an
// FP64 base point, refined in FP64 every `refine` sweeps (and at every
// residual check); F holds pgs_mixed_frows() floats per contact (mcap
// contacts), BM 8 floats and U 6 floats per body, GI one int4 per coloured
// group (ng of them)
void launch_pgs_mixed(const DBodies& B, DContacts& C, DPairs& P, const int* groupOrder, const int* colourOff,
                      int ncol, int nc, int iters, double omega, double comp, double tol, bool early, int fo,
                      double fv, double slide, double* Mj, double* K, float* F, float* BM, float* U, int4* GI,
                      int ng, int nbodies, int mcap, DCount* dc, int gridBlocks, int mode, cudaStream_t s,
                      double resTol, int check, int refine);
int pgs_mixed_frows();
// blocks of the grid form for a widest colour of `widest` groups
int pgs_mixed_grid_blocks(int widest, int coopBlocks);
// the form of the mixed solve for these colours: 0, a cooperative grid of
// gridBlocks 128-thread blocks; 1, one 256-thread block (block barriers, body
// data and delta-v corrections in shared memory); 2, one block with the
// contact records in shared memory too
int pgs_mixed_mode(const std::vector<int>& colOff, int gridBlocks, int nbodies, int nc);
// whether form `mode` of the mixed solve fits these sizes (shared memory)
bool pgs_mixed_fits(int mode, const std::vector<int>& colOff, int nbodies, int nc);
// rows of the coloured solve's per-contact constant table (1/(D+c), A, q,
// couplings, friction coefficient), each `mcap` doubles
int pgs_fast_krows();
void launch_residual(const DBodies& B, DContacts& C, int nc, double comp, int frictionOv, double frictionVal,
                     DCount* dc, cudaStream_t s);
void launch_bpc_keep(const DContacts& C, DPairs& P, int npairs, cudaStream_t s);
// a grid barrier that can never complete (its target counts one block more
// than the grid holds), bounded by 2^spin_log2 polls: every block must give
// up with AM_E_TIMEOUT in the status word and return
void launch_barrier_timeout_check(DCount* dc, int spin_log2, cudaStream_t s);

}  // namespace am
