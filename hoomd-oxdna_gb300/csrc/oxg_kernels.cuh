// oxg_kernels.cuh - sm_103a kernels of the oxDNA force engine.
//
//  k_forces          one launch per step for every force: a grid-stride loop over
//                    [short-range pairs | bonds | long-range (Debye-only) pairs],
//                    parameters staged in shared memory, float4 vector atomics
//                    (red.global.add.v4.f32) for both ends, FP64 per-term energies
//                    reduced by warp shuffles and one atomic per warp.
//  k_pairs_hoomd     the evaluator-level drop-in over a HOOMD full neighbour list:
//                    one warp per particle, lanes over neighbours, warp-shuffle
//                    force/torque reductions (no atomics), FP64 energies.
//  k_bonds_dropin    the bonded drop-in: one thread per bond, FENE in FP64.
//  k_nlist_bin / k_nlist_pairs   cell list + half pair lists split by range.
//  k_step_one / k_step_two       Langevin + NO_SQUISH (Miller et al. 2002).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "oxg_device.cuh"
#include "oxg_mlp.cuh"
#include "oxg_params.h"

namespace oxg {

// device status bits (OR-ed into Status::flags)
enum : uint32_t {
    kStCellOverflow = 1u,
    kStPairOverflow = 2u,
    kStBadIndex = 4u,
    kStNonFinite = 8u,
    kStBarrierTimeout = 32u,  // a grid-barrier wait of the persistent run kernel gave up
};

// device-resident bookkeeping of one system
struct DevStatus {
    uint32_t flags;        // kSt* bits
    uint32_t rebuild;      // neighbour list must be rebuilt this step
    uint32_t gen;          // neighbour list generation (parity selects the cell buffer)
    uint32_t n_short;      // short-range pair count
    uint32_t n_long;       // long-range pair count
    uint32_t builds;       // neighbour list builds so far
    uint32_t max_cell;     // largest cell occupancy seen
    uint32_t moved;        // run start: a particle moved half the buffer since the last build
    unsigned long long step;  // current timestep (RNG counter)
    uint32_t qcount[8];    // deferred-term queue lengths, kNQ used (k_forces_a -> k_forces_b)
    uint32_t qspill;       // run kernel: a block's shared-memory queue overflowed this step
    uint32_t rb[2];        // run kernel: rebuild requests of the next bodies, by body parity
    uint32_t changed;      // run start from host state: it differs from the device state
    uint32_t spec_far;     // run start: a particle's first step one (taken in the run start's
                           // pass) moved it half the buffer since the last build
    uint32_t seq;          // host-mapped copy only: the sequence number of the launch that
                           // wrote it, stored after every other word (never set on the device)
};

// ------------------------------------------------------------ parameter view
struct ParamView {
    const unsigned char* b;
    __device__ __forceinline__ const ParamHeader& h() const { return *reinterpret_cast<const ParamHeader*>(b); }
    template <class T>
    __device__ __forceinline__ const T& term(int t, int pidx) const
    {
        const ParamHeader& H = h();
        return *reinterpret_cast<const T*>(b + H.off[t] + pidx * H.stride[t]);
    }
    __device__ __forceinline__ const DBonded& bonded(int bt) const
    {
        return reinterpret_cast<const DBonded*>(b + h().off_bonded)[bt];
    }
};

// Copy the parameter block into dynamic shared memory (16-byte vectors).
__device__ __forceinline__ ParamView stage_params(const unsigned char* g, int bytes)
{
    extern __shared__ float4 smem_params[];
    const float4* src = reinterpret_cast<const float4*>(g);
    for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) smem_params[k] = src[k];
    __syncthreads();
    ParamView v;
    v.b = reinterpret_cast<const unsigned char*>(smem_params);
    return v;
}

// ------------------------------------------------------------ pair evaluation
// All selected nonbonded terms for one pair. dr = r_i - r_j (minimum image), E[t]
// receives each term's pair energy. Returns true if anything was non-zero.
__device__ __forceinline__ bool eval_pair(const ParamView& P, uint32_t mask, int pidx,
                                          float3 dr, float rsq, float4 qi, float4 qj,
                                          float ci, float cj, PairAcc& acc, float* E)
{
    const ParamHeader& H = P.h();
    if (!(rsq < H.rcutsq_max)) return false;
    const Frame fi = quat_frame(qi), fj = quat_frame(qj);
    const float3 rc = -dr;
    bool any = false;
    if (mask & (1u << kExcVol)) {
        const DExcVol& p = P.term<DExcVol>(kExcVol, pidx);
        if (rsq < p.rcutsq) {
            const float e = excvol_term(p, rc, fi, fj, acc);
            E[kExcVol] += e;
            any = true;
        }
    }
    if (mask & ((1u << kHBond) | (1u << kCross))) {
        const bool use_hb = (mask >> kHBond) & 1u, use_cs = (mask >> kCross) & 1u;
        const DHBond* ph = use_hb ? &P.term<DHBond>(kHBond, pidx) : nullptr;
        const DCross* pc = use_cs ? &P.term<DCross>(kCross, pidx) : nullptr;
        const bool in_hb = use_hb && rsq < ph->rcutsq;
        const bool in_cs = use_cs && rsq < pc->rcutsq;
        BBGeom g;
        bool gv = false;
        if (in_hb) {
            gv = bb_geometry(rc, fi, fj, ph->base, g);
            if (gv) {
                RadialF1 R{ph->f1, H.hb_eps[pidx], H.hb_shift[pidx]};
                E[kHBond] += bb_term<false>(g, fi, fj, ph->t1, ph->t23, ph->t4, ph->t78, true, R, acc);
            }
            any = true;
        }
        if (in_cs) {
            if (!in_hb || !H.hb_cs_same_site) gv = bb_geometry(rc, fi, fj, pc->base, g);
            if (gv) {
                RadialF2 R{pc->f2};
                E[kCross] += bb_term<true>(g, fi, fj, pc->t1, pc->t23, pc->t4, pc->t78,
                                           pc->t4_enabled != 0, R, acc);
            }
            any = true;
        }
    }
    if (mask & (1u << kHBCross)) {
        const DHBCross& p = P.term<DHBCross>(kHBCross, pidx);
        if (rsq < p.rcutsq) {
            BBGeom g;
            if (bb_geometry(rc, fi, fj, p.base, g)) {
                RadialF1 R1{p.f1, H.hbx_eps[pidx], H.hbx_shift[pidx]};
                float e = bb_term<false>(g, fi, fj, p.hb_t1, p.hb_t23, p.hb_t4, p.hb_t78, true, R1, acc);
                RadialF2 R2{p.f2};
                e += bb_term<true>(g, fi, fj, p.cs_t1, p.cs_t23, p.cs_t4, p.cs_t78, true, R2, acc);
                E[kHBCross] += e;
            }
            any = true;
        }
    }
    if (mask & (1u << kCoax)) {
        const DCoax& p = P.term<DCoax>(kCoax, pidx);
        if (rsq < p.rcutsq) {
            E[kCoax] += coax_term(p, rc, fi, fj, acc);
            any = true;
        }
    }
    if (mask & (1u << kDebye)) {
        const DDebye& p = P.term<DDebye>(kDebye, pidx);
        if (rsq < p.rcutsq) {
            E[kDebye] += debye_term(p, rc, fi, fj, ci, cj, acc);
            any = true;
        }
    }
    return any;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float3 min_image(float3 d, float3 L, float3 invL)
{
    d.x -= L.x * rintf(d.x * invL.x);
    d.y -= L.y * rintf(d.y * invL.y);
    d.z -= L.z * rintf(d.z * invL.z);
    return d;
}

__device__ __forceinline__ int type_of(float4 p) { return __float_as_int(p.w); }

// r_i - r_j from double-float positions (hi + lo): the high parts of nearby particles
// subtract almost exactly, so dr keeps ~1e-7 absolute precision in a 230-sigma box.
// r_i - r_j, minimum image, from double-float positions. The periodic shift L n is
// added to hi_j first, with the rounding error of that sum recovered exactly (TwoSum),
// so that hi_i - (hi_j + L n) is exact (Sterbenz: for a pair across the boundary of a
// box wrapped to [-L/2, L/2) both lie within a factor of two) and every low-order part
// is kept. Shifting the difference instead would round it at the ulp of L (4e-6 for
// L = 100), an error that shows as forces of ~1e-3 at the stationary points of the
// hydrogen-bonding potential.
__device__ __forceinline__ float image_axis(float hi_i, float lo_i, float hi_j, float lo_j, float L, float invL)
{
    const float n = rintf((hi_i - hi_j) * invL);
    const float Ln = L * n;  // exact: n is -1, 0 or 1 for positions in the box
    const float s = hi_j + Ln;
    const float bb = s - hi_j;
    const float err = (hi_j - (s - bb)) + (Ln - bb);  // hi_j + Ln = s + err exactly
    return (hi_i - s) + ((lo_i - lo_j) - err);
}
__device__ __forceinline__ float3 image_delta(float4 hi_i, float4 lo_i, float4 hi_j, float4 lo_j, float3 L, float3 invL)
{
    return mk3(image_axis(hi_i.x, lo_i.x, hi_j.x, lo_j.x, L.x, invL.x),
               image_axis(hi_i.y, lo_i.y, hi_j.y, lo_j.y, L.y, invL.y),
               image_axis(hi_i.z, lo_i.z, hi_j.z, lo_j.z, L.z, invL.z));
}

// ----------------------------------------------------------- engine force kernel
struct ForceArgs {
    const unsigned char* params;
    int param_bytes;
    uint32_t mask;        // nonbonded terms
    int bonded;           // evaluate bonds
    int N;
    int n_bonds;
    const float4* pos;    // x, y, z (high parts), type bits
    const float4* pos_lo; // low parts of x, y, z (double-float positions)
    const float4* quat;
    const float* charge;
    const int4* bonds;    // A, B, type, unused
    const int2* pairs_short;
    const int2* pairs_long;
    const DevStatus* st;  // n_short / n_long
    DevStatus* st_rw;     // rebuild flag cleared here
    int cap_short, cap_long;  // list capacities (counts past them were not stored)
    int advance_step;     // MD step: advance the RNG step counter read by step two
    int2* queue;          // kNQ deferred-term queues of cap_short pairs (i, j)
    float3 L, invL;
    float4* force;        // accumulated (pre-zeroed)
    float4* torque;
    double* energy;       // [6 pair terms][3 bonded] (ENERGY only)
    float* virial;        // unused by the engine
    // learned surrogate of the fused HB + cross-stacking term (null: plain evaluator)
    const MlpDev* mlp = nullptr;
    struct SurrogateAudit* audit = nullptr;
    uint32_t audit_every = 0;  // steps between audits (0: never)
    uint32_t audit_mod = 100;  // one queued pair in audit_mod is audited
    float audit_tol = 1e-4f;   // largest accepted relative error of the term's energy
    // entries per heavy-term queue a block keeps in shared memory in phase A (at most
    // kBlockQ; lowered only to exercise the path of pairs that do not fit)
    int block_q = 400;
};

// Statistics of the audits of the surrogate by the plain evaluator; `disabled` is the
// kill switch the force kernels read. The audited pairs are a hashed sample of the
// term's pairs, so sum_de / sum_e estimates the relative error of the term's energy;
// the switch trips when that estimate exceeds the tolerance by more than two standard
// errors (at least kAuditMinPairs audited pairs), tested by the next step's forces A
// (audit_decide below), which sets `disabled`, so every kernel of a step sees the same
// switch.
struct SurrogateAudit {
    uint32_t disabled;           // read by the force kernels; set at a step start
    uint32_t n_audited;
    uint32_t n_over;             // step starts at which the test failed (at most 1)
    uint32_t pending;            // the test has failed
    double sum_sq_de, sum_sq_e;  // pair energy error and reference
    double sum_sq_df, sum_sq_f;  // force (on i) error and reference
    double sum_de, sum_e;        // signed sums of the pair energy error and reference
    float max_abs_de, max_abs_df;
    float pad2[2];
};
constexpr uint32_t kAuditMinPairs = 100;

// The kill switch, decided at a step start (block 0 of the step's first kernel, so that
// every kernel of the step sees one value) from the complete sums of every audit so far:
// the sampled relative error of the term's energy above the tolerance by more than two
// standard errors, over at least kAuditMinPairs pairs (a NaN trips it too). Testing the
// running sums after each audited pair instead tripped on partial samples: pairs are
// audited in queue order, class by class, and the first hundreds of one class carry that
// class's error against its own smaller energy sum.
__device__ __forceinline__ void audit_decide(SurrogateAudit* au, float tol)
{
    if (au->disabled) return;
    const uint32_t n = au->n_audited;
    const double se = au->sum_e;
    if (n < kAuditMinPairs || se == 0.0) return;
    const double mean = au->sum_de / n;
    const double se_rel = sqrt(fmax(au->sum_sq_de / n - mean * mean, 0.0) * n) / fabs(se);
    const double rel = fabs(au->sum_de) / fabs(se);
    if (!(rel - 2.0 * se_rel <= (double)tol)) {
        au->disabled = 1u;
        au->pending = 1u;
        au->n_over += 1u;
    }
}

// The force evaluation is split in two launches so that the acos-heavy terms run with
// every lane busy (whatever the system size):
//  k_forces_a  one thread per short-range pair evaluates the cheap terms (excluded
//              volume, Debye) and the zero-factor tests of the heavy ones (HB,
//              cross-stacking, fused HB+CS, coaxial stacking), appending each pair that
//              passes to that term's queue (warp-aggregated atomics); then the
//              long-range (Debye-only) pairs;
//  k_forces_b  term-uniform warps over [HB | CS | HB+CS | coax | bonds]: each warp
//              evaluates 32 queued pairs (or bonds) of one term.
// The integrator kernels reset the queue lengths for the next step.
// The fused HB + cross-stacking pairs are queued by class (complementary bases in kQHBX,
// the rest in kQHBX0) so that a warp of the surrogate evaluates one network.
enum { kQHB = 0, kQCS = 1, kQHBX = 2, kQCX = 3, kQHBX0 = 4, kNQ = 5 };

struct PairIn {
    int i, j, pidx;
    float3 rc;  // r_j - r_i
    float rsq;
    float ci, cj;
    float4 qi, qj;  // orientations (loaded with the positions: one L2 round trip)
};

__device__ __forceinline__ bool load_pair(const ForceArgs& a, int2 pr, int n_types, PairIn& p,
                                          bool& bad_type)
{
    p.i = pr.x;
    p.j = pr.y;
    // every load of the pair issued at once (one L2 round trip)
    const float4 pi = __ldcg(a.pos + p.i), pj = __ldcg(a.pos + p.j);
    const float4 li = __ldcg(a.pos_lo + p.i), lj = __ldcg(a.pos_lo + p.j);
    p.qi = __ldcg(a.quat + p.i);
    p.qj = __ldcg(a.quat + p.j);
    const float3 dr = image_delta(pi, li, pj, lj, a.L, a.invL);
    p.rc = -dr;
    p.rsq = dot(dr, dr);
    const int ti = type_of(pi), tj = type_of(pj);
    if ((unsigned)ti >= (unsigned)n_types || (unsigned)tj >= (unsigned)n_types) {
        bad_type = true;
        return false;
    }
    p.pidx = ti * kMaxTypes + tj;
    p.ci = a.charge ? a.charge[p.i] : 1.f;
    p.cj = a.charge ? a.charge[p.j] : 1.f;
    return true;
}
template <bool ENERGY>
__device__ __forceinline__ void scatter(const ForceArgs& a, int i, int j, const PairAcc& acc, float e)
{
    const float eh = ENERGY ? 0.5f * e : 0.f;
    atomicAdd(a.force + i, make_float4(acc.fi.x, acc.fi.y, acc.fi.z, eh));
    atomicAdd(a.force + j, make_float4(-acc.fi.x, -acc.fi.y, -acc.fi.z, eh));
    atomicAdd(a.torque + i, make_float4(acc.ti.x, acc.ti.y, acc.ti.z, 0.f));
    atomicAdd(a.torque + j, make_float4(acc.tj.x, acc.tj.y, acc.tj.z, 0.f));
}

// The forces of a unit's pairs with the i side summed over each run of adjacent lanes
// with equal i (the lists hold a particle's pairs mostly contiguously) by a segmented
// suffix sum over the warp: the run's first lane adds the run's total with one atomic
// per array, instead of one per pair; the j side is added per pair. A particle whose
// pairs are split over runs that are not adjacent (list appends of other warps in
// between) is added once per run. key: the pair's i, or -1 for a lane outside the list;
// has: the lane's pair contributed (acc, e valid). All lanes call it.
// (8000 nt: phase A 6.0 -> 5.45 us, 59.5k -> 61.0k steps/s; 100k nt: 11.5k -> 12.1k.)
template <bool ENERGY>
__device__ __forceinline__ void scatter_seg(const ForceArgs& a, int key, bool has, int i, int j,
                                            const PairAcc& acc, float e)
{
    const int lane = threadIdx.x & 31;
    const float eh = ENERGY ? 0.5f * e : 0.f;
    // force, energy half, torque, and the count of contributing pairs of the run
    float v[8] = {acc.fi.x, acc.fi.y, acc.fi.z, eh, acc.ti.x, acc.ti.y, acc.ti.z, 1.f};
#pragma unroll
    for (int c = 0; c < 8; ++c)
        if (!has) v[c] = 0.f;
    // run heads: lanes whose left neighbour has another key; a run ends before the next head
    const int kp = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || kp != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned above = heads & ~((2u << lane) - 1u);  // heads right of this lane
    const int end = above ? __ffs(above) - 2 : 31;       // last lane of this lane's run
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const bool add = lane + off <= end;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float o = __shfl_down_sync(0xffffffffu, v[c], off);
            if (add) v[c] += o;
        }
    }
    if (head && key >= 0 && v[7] > 0.f) {
        atomicAdd(a.force + i, make_float4(v[0], v[1], v[2], v[3]));
        atomicAdd(a.torque + i, make_float4(v[4], v[5], v[6], 0.f));
    }
    if (has) {
        atomicAdd(a.force + j, make_float4(-acc.fi.x, -acc.fi.y, -acc.fi.z, eh));
        atomicAdd(a.torque + j, make_float4(acc.tj.x, acc.tj.y, acc.tj.z, 0.f));
    }
}

// Full evaluation of one deferred term for short pair w (warp-uniform q). part (fused
// HB + CS pairs only): 0 both terms, 1 the HB term, 2 the CS term.
template <bool ENERGY>
__device__ __forceinline__ void eval_deferred(const ForceArgs& a, const ParamView& P, int q, int2 pr,
                                              double* eacc, int part = 0)
{
    const ParamHeader& H = P.h();
    PairIn p;
    bool dummy = false;
    if (!load_pair(a, pr, H.n_types, p, dummy)) return;
    const Frame fi = quat_frame(p.qi), fj = quat_frame(p.qj);
    PairAcc acc;
    acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
    float e = 0.f;
    int term = kHBond;
    BBGeom g;
    if (q == kQHB) {
        const DHBond& ph = P.term<DHBond>(kHBond, p.pidx);
        if (bb_geometry(p.rc, fi, fj, ph.base, g)) {
            RadialF1 R{ph.f1, H.hb_eps[p.pidx], H.hb_shift[p.pidx]};
            e = bb_term<false>(g, fi, fj, ph.t1, ph.t23, ph.t4, ph.t78, true, R, acc);
        }
    } else if (q == kQCS) {
        term = kCross;
        const DCross& pc = P.term<DCross>(kCross, p.pidx);
        if (bb_geometry(p.rc, fi, fj, pc.base, g)) {
            RadialF2 R{pc.f2};
            e = bb_term<true>(g, fi, fj, pc.t1, pc.t23, pc.t4, pc.t78, pc.t4_enabled != 0, R, acc);
        }
    } else if (q == kQHBX || q == kQHBX0) {
        term = kHBCross;
        const DHBCross& px = P.term<DHBCross>(kHBCross, p.pidx);
        if (bb_geometry(p.rc, fi, fj, px.base, g)) {
            if (part != 2) {
                RadialF1 R1{px.f1, H.hbx_eps[p.pidx], H.hbx_shift[p.pidx]};
                e = bb_term<false>(g, fi, fj, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1, acc);
            }
            if (part != 1) {
                RadialF2 R2{px.f2};
                e += bb_term<true>(g, fi, fj, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2, acc);
            }
        }
    } else {
        term = kCoax;
        e = coax_term(P.term<DCoax>(kCoax, p.pidx), p.rc, fi, fj, acc);
    }
    scatter<ENERGY>(a, p.i, p.j, acc, e);
    if (ENERGY) eacc[term] += (double)e;
}

template <bool ENERGY>
__device__ __forceinline__ void reduce_energies(const ForceArgs& a, double* eacc)
{
    if (!ENERGY) return;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int t = 0; t < kNTerms + 3; ++t) {
        const double sum = warp_sum(eacc[t]);
        if (lane == 0 && sum != 0.0) atomicAdd(a.energy + t, sum);
    }
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }

// Warp `gwarp` of `nwarps`: short-range pairs in units of 32 (cheap terms inline, heavy
// ones queued), then the long-range pairs. Counters are read with volatile loads: the
// persistent run kernel calls this after a neighbour-list rebuild in the same launch.
// The long-pair units of warp gwarp: v0, v0 + vstride, ... When the short units leave
// warps free (small systems) the long units go to those warps only (a short unit costs
// about as much as three or four long ones); otherwise round-robin over all warps.
__device__ __forceinline__ void long_units(int gwarp, int nwarps, int n_short, int n_long, int& v0, int& vstride)
{
    const int n_su = (n_short + 31) >> 5, n_lu = (n_long + 31) >> 5;
    const int free_w = nwarps - n_su;
    const bool to_free = free_w > 0 && 4 * free_w >= n_lu;
    v0 = to_free ? gwarp - n_su : gwarp;
    vstride = to_free ? free_w : nwarps;
}

// Phase A appends the heavy-term pairs of a block to shared-memory queues (shared
// atomics) and copies them to the global queues at the end of the phase with one global
// atomic per queue and block, instead of one same-address global atomic per warp, term
// and unit. A reservation that does not fit goes to the global queue directly.
constexpr int kBlockQ = 400;  // entries per queue and block (the largest ForceArgs::block_q)
struct BlockQueues {
    uint32_t count[kNQ];  // reserved entries
    uint32_t valid[kNQ];  // entries below this offset were all written
    uint32_t base[kNQ];   // global offsets of the flush
    int2 buf[kNQ][kBlockQ];
};

__device__ __forceinline__ BlockQueues& block_queues()
{
    __shared__ BlockQueues bq;
    return bq;
}

// LOCAL: the block's heavy-term pairs stay in its shared-memory queues for
// forces_b_local (the run kernel); otherwise they are copied to the global queues.
// n_short_known / n_long_known: the stored pair counts when the caller has them (the run
// kernel keeps them between rebuilds), else negative: read from the status block.
// first: this thread's first short- and long-pair entries when the caller keeps them
// (with the counts), else null.
template <bool ENERGY, bool LOCAL = false>
__device__ __forceinline__ void forces_a_body(const ForceArgs& a, const ParamView& P, int gwarp,
                                              int nwarps, double* eacc, bool& bad_type,
                                              int n_short_known = -1, int n_long_known = -1,
                                              const int2* first = nullptr)
{
    BlockQueues& bq = block_queues();
    const uint32_t qcap = (uint32_t)min(max(a.block_q, 0), kBlockQ);
    if (threadIdx.x < kNQ) {
        bq.count[threadIdx.x] = 0u;
        bq.valid[threadIdx.x] = qcap;
    }
    __syncthreads();
    const ParamHeader& H = P.h();
    // after an overflow the counters exceed the capacities; only stored pairs are read
    const int n_short = n_short_known >= 0 ? n_short_known
                                           : (int)min(ld_volatile(&a.st_rw->n_short), (uint32_t)a.cap_short);
    const int n_long = n_long_known >= 0 ? n_long_known
                                         : (int)min(ld_volatile(&a.st_rw->n_long), (uint32_t)a.cap_long);
    const int n_types = H.n_types;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint32_t mask = a.mask;

    // the next unit's pair entry is loaded one unit ahead (a warp takes several units
    // of a large system: one L2 round trip of each unit's chain is hidden)
    const int stride = nwarps * 32;
    int2 next_pr = first ? first[0]
                         : (gwarp * 32 + lane < n_short ? __ldcg(a.pairs_short + gwarp * 32 + lane) : make_int2(0, 0));
    for (int base = gwarp * 32; base < n_short; base += stride) {
        const int w = base + lane;
        const int2 pr = next_pr;
        if (w + stride < n_short) next_pr = __ldcg(a.pairs_short + w + stride);
        bool want[kNQ] = {};
        PairIn p;
        PairAcc acc;
        acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
        float e_inline = 0.f;
        bool inl = false;
        if (w < n_short && load_pair(a, pr, n_types, p, bad_type) && p.rsq < H.rcutsq_max) {
            const Frame fi = quat_frame(p.qi), fj = quat_frame(p.qj);
            if (mask & (1u << kExcVol)) {
                const DExcVol& pe = P.term<DExcVol>(kExcVol, p.pidx);
                if (p.rsq < pe.rcutsq) {
                    const float e = excvol_term(pe, p.rc, fi, fj, acc);
                    e_inline += e;
                    if (ENERGY) eacc[kExcVol] += (double)e;
                    inl = true;
                }
            }
            if (mask & (1u << kDebye)) {
                const DDebye& pd = P.term<DDebye>(kDebye, p.pidx);
                if (p.rsq < pd.rcutsq) {
                    const float e = debye_term(pd, p.rc, fi, fj, p.ci, p.cj, acc);
                    e_inline += e;
                    if (ENERGY) eacc[kDebye] += (double)e;
                    inl = true;
                }
            }
            BBGeom g;
            bool gv = false;
            if (mask & (1u << kHBond)) {
                const DHBond& ph = P.term<DHBond>(kHBond, p.pidx);
                if (p.rsq < ph.rcutsq && H.hb_eps[p.pidx] != 0.f) {
                    gv = bb_geometry(p.rc, fi, fj, ph.base, g);
                    RadialF1 R{ph.f1, H.hb_eps[p.pidx], H.hb_shift[p.pidx]};
                    want[kQHB] = gv && bb_support<false>(g, ph.t1, ph.t23, ph.t4, ph.t78, true, R);
                }
            }
            if (mask & (1u << kCross)) {
                const DCross& pc = P.term<DCross>(kCross, p.pidx);
                if (p.rsq < pc.rcutsq) {
                    if (!gv || !H.hb_cs_same_site) gv = bb_geometry(p.rc, fi, fj, pc.base, g);
                    RadialF2 R{pc.f2};
                    want[kQCS] = gv && bb_support<true>(g, pc.t1, pc.t23, pc.t4, pc.t78,
                                                        pc.t4_enabled != 0, R);
                }
            }
            if (mask & (1u << kHBCross)) {
                const DHBCross& px = P.term<DHBCross>(kHBCross, p.pidx);
                if (p.rsq < px.rcutsq && bb_geometry(p.rc, fi, fj, px.base, g)) {
                    RadialF1 R1{px.f1, H.hbx_eps[p.pidx], H.hbx_shift[p.pidx]};
                    RadialF2 R2{px.f2};
                    want[H.hbx_eps[p.pidx] != 0.f ? kQHBX : kQHBX0] =
                        bb_support<false>(g, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1) ||
                        bb_support<true>(g, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2);
                }
            }
            if (mask & (1u << kCoax)) {
                const DCoax& pc = P.term<DCoax>(kCoax, p.pidx);
                want[kQCX] = p.rsq < pc.rcutsq && coax_support(pc, p.rc, fi, fj);
            }
        }
        scatter_seg<ENERGY>(a, w < n_short ? pr.x : -1, inl, p.i, p.j, acc, e_inline);
#pragma unroll
        for (int q = 0; q < kNQ; ++q) {
            const unsigned m = __ballot_sync(0xffffffffu, want[q]);
            if (m) {
                const int leader = __ffs(m) - 1;
                const uint32_t n = (uint32_t)__popc(m);
                uint32_t off = 0;
                if (lane == leader) {
                    off = atomicAdd(&bq.count[q], n);
                    if (off + n > qcap) {  // does not fit: straight to the global queue
                        if (off < qcap) atomicMin(&bq.valid[q], off);
                        off = 0x80000000u | atomicAdd(&a.st_rw->qcount[q], n);
                        if (LOCAL) a.st_rw->qspill = 1u;
                    }
                }
                off = __shfl_sync(0xffffffffu, off, leader);
                if (want[q]) {
                    const int2 e = make_int2(p.i, p.j);
                    const uint32_t k = (off & 0x7fffffffu) + __popc(m & lt_mask);
                    if (off & 0x80000000u) a.queue[(size_t)q * a.cap_short + k] = e;
                    else bq.buf[q][k] = e;
                }
            }
        }
    }

    // long-range pairs: Debye only (uniform, cheap), in units of 32. When the short units
    // leave warps free (small systems), the long units go to those warps only (a short
    // unit costs about as much as three or four long ones); otherwise round-robin.
    const uint32_t long_mask = mask & (1u << kDebye);
    int v0, vstride;
    long_units(gwarp, nwarps, n_short, n_long, v0, vstride);
    const int n_lu = (n_long + 31) >> 5;
    int2 next_lp = first ? first[1]
                         : ((v0 >= 0 && v0 * 32 + lane < n_long) ? __ldcg(a.pairs_long + v0 * 32 + lane) : make_int2(0, 0));
    for (int v = v0; v >= 0 && v < n_lu && long_mask; v += vstride) {
        const int w = v * 32 + lane;
        const int2 pr = next_lp;
        if (w + vstride * 32 < n_long) next_lp = __ldcg(a.pairs_long + w + vstride * 32);
        const int i = pr.x, j = pr.y;
        const bool in_range = w < n_long;
        // every load of the pair issued at once (one L2 round trip)
        const float4 pi = __ldcg(a.pos + i), pj = __ldcg(a.pos + j);
        const float4 li = __ldcg(a.pos_lo + i), lj = __ldcg(a.pos_lo + j);
        const float4 qi = __ldcg(a.quat + i), qj = __ldcg(a.quat + j);
        const float ci = a.charge ? a.charge[i] : 1.f, cj = a.charge ? a.charge[j] : 1.f;
        const int ti = type_of(pi), tj = type_of(pj);
        const bool tok = (unsigned)ti < (unsigned)n_types && (unsigned)tj < (unsigned)n_types;
        if (in_range && !tok) bad_type = true;
        const float3 dr = image_delta(pi, li, pj, lj, a.L, a.invL);
        PairAcc acc;
        acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
        float E[kNTerms] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        bool has = false;
        if (in_range && tok && eval_pair(P, long_mask, ti * kMaxTypes + tj, dr, dot(dr, dr), qi, qj, ci, cj, acc, E)) {
            if (ENERGY) eacc[kDebye] += (double)E[kDebye];
            has = true;
        }
        scatter_seg<ENERGY>(a, in_range ? i : -1, has, i, j, acc, E[kDebye]);
    }
    __syncthreads();
    if (LOCAL) {  // the entries written, for forces_b_local after the block's barrier
        if (threadIdx.x < kNQ) bq.count[threadIdx.x] = min(bq.count[threadIdx.x], bq.valid[threadIdx.x]);
        __syncthreads();
        return;
    }
    // the block's staged heavy-term pairs to the global queues
    if (threadIdx.x < kNQ) {
        const uint32_t n = min(bq.count[threadIdx.x], bq.valid[threadIdx.x]);
        bq.count[threadIdx.x] = n;
        bq.base[threadIdx.x] = n ? atomicAdd(&a.st_rw->qcount[threadIdx.x], n) : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kNQ; ++q) {
        const uint32_t n = bq.count[q], b = bq.base[q];
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
            if (b + k < (uint32_t)a.cap_short) a.queue[(size_t)q * a.cap_short + b + k] = bq.buf[q][k];
    }
}

// Warps interleaved across the blocks (warp w of block b is unit w * gridDim + b), so
// that a short list of work units is spread over every SM rather than the first blocks.
__device__ __forceinline__ int spread_warp() { return (threadIdx.x >> 5) * gridDim.x + blockIdx.x; }

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_forces_a(ForceArgs a)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.st_rw->rebuild) {
            a.st_rw->rebuild = 0u;
            a.st_rw->gen += 1u;
        }
        if (a.advance_step) a.st_rw->step += 1ull;
        // the audits so far decide whether the surrogate stays on for this step
        if (a.audit) audit_decide(a.audit, a.audit_tol);
    }
    double eacc[kNTerms + 3];
#pragma unroll
    for (int t = 0; t < kNTerms + 3; ++t) eacc[t] = 0.0;
    bool bad_type = false;
    forces_a_body<ENERGY>(a, P, spread_warp(), (gridDim.x * blockDim.x) >> 5, eacc, bad_type);
    reduce_energies<ENERGY>(a, eacc);
    if (bad_type) atomicOr(&a.st_rw->flags, kStBadIndex);
}

// ------------------------------------------------------------ surrogate path
// Plain evaluation of an audited pair next to the surrogate's: energy and force errors
// into the statistics, and the kill switch when the energy error exceeds the tolerance.
static __device__ __noinline__ void surrogate_audit(const ForceArgs& a, const ParamView& P, int pidx,
                                             const BBGeom& g, const Frame& fi, const Frame& fj,
                                             float e_sur, const PairAcc& acc_sur)
{
    const ParamHeader& H = P.h();
    const DHBCross& px = P.term<DHBCross>(kHBCross, pidx);
    PairAcc pa;
    pa.fi = pa.ti = pa.tj = mk3(0.f, 0.f, 0.f);
    RadialF1 R1{px.f1, H.hbx_eps[pidx], H.hbx_shift[pidx]};
    float e = bb_term<false>(g, fi, fj, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1, pa);
    RadialF2 R2{px.f2};
    e += bb_term<true>(g, fi, fj, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2, pa);
    const float de = e_sur - e;
    const float3 df = acc_sur.fi - pa.fi;
    const float df2 = dot(df, df);
    SurrogateAudit* au = a.audit;
    atomicAdd(&au->n_audited, 1u);
    atomicAdd(&au->sum_sq_de, (double)de * de);
    atomicAdd(&au->sum_sq_e, (double)e * e);
    atomicAdd(&au->sum_sq_df, (double)df2);
    atomicAdd(&au->sum_sq_f, (double)dot(pa.fi, pa.fi));
    atomicAdd(&au->sum_de, (double)de);
    atomicAdd(&au->sum_e, (double)e);
    // non-negative floats order like their bit patterns
    atomicMax(reinterpret_cast<int*>(&au->max_abs_de), __float_as_int(fabsf(de)));
    atomicMax(reinterpret_cast<int*>(&au->max_abs_df), __float_as_int(sqrtf(df2)));
}

__device__ __forceinline__ bool audit_pick(int k, unsigned long long step, uint32_t mod)
{
    const uint32_t h = ((uint32_t)k * 2654435761u) ^ ((uint32_t)step * 40503u + 0x9e3779b9u);
    return (h % mod) == 0u;
}

// One bond (part: 0 whole, 1 FENE + bonded excluded volume, 2 stacking).
template <bool ENERGY>
__device__ __forceinline__ void eval_bond(const ForceArgs& a, const ParamView& P, int4 bd, int n_types,
                                          double* eacc, bool& bad_type, int part)
{
    const int A = bd.x, B = bd.y;
    const float4 pA = __ldcg(a.pos + A), pB = __ldcg(a.pos + B);
    if ((unsigned)type_of(pA) >= (unsigned)n_types || (unsigned)type_of(pB) >= (unsigned)n_types) {
        bad_type = true;
        return;
    }
    const float3 Rcf = image_delta(pB, __ldcg(a.pos_lo + B), pA, __ldcg(a.pos_lo + A), a.L, a.invL);
    const float4 qA = __ldcg(a.quat + A), qB = __ldcg(a.quat + B);
    const double3 Rc = make_double3(Rcf.x, Rcf.y, Rcf.z);
    const double4_32a dA = make_double4_32a(qA.x, qA.y, qA.z, qA.w), dB = make_double4_32a(qB.x, qB.y, qB.z, qB.w);
    BondAcc acc;
    if (part == 1) bonded_pair<false, 1>(P.bonded(bd.z), Rc, dA, dB, type_of(pA), type_of(pB), acc);
    else if (part == 2) bonded_pair<false, 2>(P.bonded(bd.z), Rc, dA, dB, type_of(pA), type_of(pB), acc);
    else bonded_pair<false>(P.bonded(bd.z), Rc, dA, dB, type_of(pA), type_of(pB), acc);
    float eh = 0.f;
    if (ENERGY) {
        eacc[kNTerms + 0] += acc.e[0];
        eacc[kNTerms + 1] += acc.e[1];
        eacc[kNTerms + 2] += acc.e[2];
        eh = (float)(0.5 * (acc.e[0] + acc.e[1] + acc.e[2]));
    }
    atomicAdd(a.force + A, make_float4(-acc.fB.x, -acc.fB.y, -acc.fB.z, eh));
    atomicAdd(a.force + B, make_float4(acc.fB.x, acc.fB.y, acc.fB.z, eh));
    atomicAdd(a.torque + A, make_float4(acc.tA.x, acc.tA.y, acc.tA.z, 0.f));
    atomicAdd(a.torque + B, make_float4(acc.tB.x, acc.tB.y, acc.tB.z, 0.f));
}

// Warp `gwarp` of `nwarps` over the segments [HB | CS | HB+CS | coax | HB+CS (other) |
// bonds], each padded to whole warps: every warp evaluates 32 items of one term.
// (Evaluating the bonds on two lanes each, FENE + bonded excluded volume | stacking,
// shortens their chains but not the phase: the HB and cross-stacking items are as long.)
template <bool ENERGY, bool BONDS = true>
__device__ __forceinline__ void forces_b_body(const ForceArgs& a, const ParamView& P, int gwarp,
                                              int nwarps, double* eacc, bool& bad_type)
{
    const int n_types = P.h().n_types;
    int cnt[kNQ + 1], seg[kNQ + 2];
    seg[0] = 0;
#pragma unroll
    for (int q = 0; q < kNQ; ++q) cnt[q] = (int)min(ld_volatile(&a.st_rw->qcount[q]), (uint32_t)a.cap_short);
    cnt[kNQ] = (BONDS && a.bonded) ? a.n_bonds : 0;
#pragma unroll
    for (int q = 0; q <= kNQ; ++q) seg[q + 1] = seg[q] + ((cnt[q] + 31) & ~31);
    const int lane = threadIdx.x & 31;
    // the fused HB + CS queues are the surrogate kernel's while it is switched on
    if (a.mlp != nullptr && ld_volatile(&a.audit->disabled) == 0u) cnt[kQHBX] = cnt[kQHBX0] = 0;
#pragma unroll
    for (int q = 0; q <= kNQ; ++q) seg[q + 1] = seg[q] + ((cnt[q] + 31) & ~31);
    for (int wbase = gwarp * 32; wbase < seg[kNQ + 1]; wbase += nwarps * 32) {
        int q = 0;
        while (q < kNQ && wbase >= seg[q + 1]) ++q;  // warp-uniform segment
        const int k = wbase - seg[q] + lane;
        if (k >= cnt[q]) continue;
        if (q < kNQ) eval_deferred<ENERGY>(a, P, q, __ldcg(a.queue + (size_t)q * a.cap_short + k), eacc);
        else eval_bond<ENERGY>(a, P, a.bonds[k], n_types, eacc, bad_type, 0);
    }
}

// Phase B of a block on its own shared-memory queues (filled by forces_a_body<.., true>
// of the same block: no grid barrier between the phases) and its share of the bonds,
// 32 items of one term per warp.
// bond_stage: the block's slice of the bonds in shared memory (or null: read the global
// table). The slice is [n_bonds * block / grid, n_bonds * (block + 1) / grid).
template <bool ENERGY>
__device__ __forceinline__ void forces_b_local(const ForceArgs& a, const ParamView& P, double* eacc,
                                               bool& bad_type, const int4* bond_stage = nullptr)
{
    BlockQueues& bq = block_queues();
    const int n_types = P.h().n_types;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nb = a.bonded ? a.n_bonds : 0;
    const int b0 = (int)((long long)nb * blockIdx.x / gridDim.x);
    const int b1 = (int)((long long)nb * (blockIdx.x + 1) / gridDim.x);
    // segments: the kNQ queues, then the cross-stacking halves of the fused HB + CS pairs
    // of complementary bases (their queue segment takes the HB halves: two items of one
    // term each instead of one of both), then the bonds; the fused pairs of the other
    // class take the CS half only (their HB factor is zero: the half adds exactly zero)
    int cnt[kNQ + 2], seg[kNQ + 3];
    seg[0] = 0;
#pragma unroll
    for (int q = 0; q < kNQ; ++q) cnt[q] = (int)bq.count[q];
    cnt[kNQ] = cnt[kQHBX];
    cnt[kNQ + 1] = b1 - b0;
#pragma unroll
    for (int q = 0; q <= kNQ + 1; ++q) seg[q + 1] = seg[q] + ((cnt[q] + 31) & ~31);
    for (int wbase = w * 32; wbase < seg[kNQ + 2]; wbase += nw * 32) {
        int q = 0;
        while (q < kNQ + 1 && wbase >= seg[q + 1]) ++q;  // warp-uniform segment
        const int k = wbase - seg[q] + lane;
        if (k >= cnt[q]) continue;
        if (q < kNQ) {
            const int part = q == kQHBX ? 1 : (q == kQHBX0 ? 2 : 0);
            eval_deferred<ENERGY>(a, P, q, bq.buf[q][k], eacc, part);
        } else if (q == kNQ) {
            eval_deferred<ENERGY>(a, P, kQHBX, bq.buf[kQHBX][k], eacc, 2);
        } else {
            eval_bond<ENERGY>(a, P, bond_stage ? bond_stage[k] : a.bonds[b0 + k], n_types, eacc, bad_type, 0);
        }
    }
}

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_forces_b(ForceArgs a)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    double eacc[kNTerms + 3];
#pragma unroll
    for (int t = 0; t < kNTerms + 3; ++t) eacc[t] = 0.0;
    bool bad_type = false;
    forces_b_body<ENERGY>(a, P, spread_warp(), (gridDim.x * blockDim.x) >> 5, eacc, bad_type);
    reduce_energies<ENERGY>(a, eacc);
    if (bad_type) atomicOr(&a.st_rw->flags, kStBadIndex);
}

// ------------------------------------------------------ surrogate (tcgen05)
// The queued fused HB + cross-stacking pairs of both classes through the surrogate
// network on the tensor cores, 128 pairs per tile, a pair per thread of a 128-thread
// block: features from the plain evaluator's base-base geometry, energy and input
// gradient from the network (tc_rows128), forces and torques from the gradient,
// scattered like the plain evaluator's; on audit steps a hashed sample of the pairs is
// also evaluated by the plain evaluator. It runs between forces A (which queued the
// pairs) and forces B (which leaves these queues to it while the surrogate is on).
// Dynamic shared memory: the parameter block, then one class's weight image and the
// tile's operand buffers; blocks take tiles [class 1 | class 0] round robin and load the
// weights of a class when they first meet it.
constexpr int kSurrThreads = 128;
constexpr uint32_t kSurrW = 0, kSurrX = tc::kImgBytes, kSurrP = kSurrX + kTcX, kSurrQ = kSurrP + kTcAct,
                   kSurrBuf = kSurrQ + kTcAct;
// at least 80 KB per block so that at most two blocks (2 x 256 tensor-memory columns) share an SM
__host__ __device__ constexpr uint32_t surrogate_smem(int param_bytes)
{
    const uint32_t need = (((uint32_t)param_bytes + 1023u) & ~1023u) + kSurrBuf;
    return need > 81920u ? need : 81920u;
}

template <bool ENERGY>
__global__ void __launch_bounds__(kSurrThreads) k_surrogate(ForceArgs a)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    extern __shared__ float4 smem_params[];
    unsigned char* buf = reinterpret_cast<unsigned char*>(smem_params) + (((uint32_t)a.param_bytes + 1023u) & ~1023u);
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    if (ld_volatile(&a.audit->disabled)) return;  // switched off (constant during the step)
    const int tid = threadIdx.x, warp = tid >> 5;
    const ParamHeader& H = P.h();
    const int n1 = (int)min(ld_volatile(&a.st_rw->qcount[kQHBX]), (uint32_t)a.cap_short);
    const int n0 = (int)min(ld_volatile(&a.st_rw->qcount[kQHBX0]), (uint32_t)a.cap_short);
    const int t1 = (n1 + kTcRows - 1) / kTcRows, t0 = (n0 + kTcRows - 1) / kTcRows;
    if ((int)blockIdx.x >= t1 + t0) return;
    if (warp == 0) tc::tmem_alloc(tc::smem_addr(&tmem_base), 256);
    if (tid == 0) tc::mbar_init(tc::smem_addr(&mbar), 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    TcTile t;
    t.w = buf + kSurrW;
    t.x = buf + kSurrX;
    t.p = buf + kSurrP;
    t.q = buf + kSurrQ;
    t.mbar = tc::smem_addr(&mbar);
    t.tmem = tmem_base;
    t.bar_id = 1;
    const unsigned long long step = *(const volatile unsigned long long*)&a.st_rw->step;
    const bool audit_step = a.audit_every != 0u && (step % a.audit_every) == 0ull;
    double eacc[kNTerms + 3];
#pragma unroll
    for (int k = 0; k < kNTerms + 3; ++k) eacc[k] = 0.0;
    uint32_t phase = 0;
    int loaded = -1;
    bool ok = true;
    for (int tile = blockIdx.x; tile < t1 + t0 && ok; tile += gridDim.x) {
        const int cls = tile < t1 ? 1 : 0;
        const int q = cls ? kQHBX : kQHBX0;
        const int k = (cls ? tile : tile - t1) * kTcRows + tid;
        if (cls != loaded) {  // block-uniform; the previous tile's MMAs have completed
            tc_load_weights(t.w, a.mlp->tcw[cls]);
            loaded = cls;
        }
        const MlpVec& V = a.mlp->vec[cls];
        PairIn p;
        BBGeom g;
        Frame fi, fj;
        float x[kMlpIn];
#pragma unroll
        for (int f = 0; f < kMlpIn; ++f) x[f] = 0.f;
        bool valid = k < (cls ? n1 : n0);
        if (valid) {
            bool bad = false;
            valid = load_pair(a, __ldcg(a.queue + (size_t)q * a.cap_short + k), H.n_types, p, bad);
            if (valid) {
                fi = quat_frame(p.qi);
                fj = quat_frame(p.qj);
                valid = bb_geometry(p.rc, fi, fj, P.term<DHBCross>(kHBCross, p.pidx).base, g);
            }
            if (valid) {
                mlp_features(g, x);
#pragma unroll
                for (int f = 0; f < kMlpIn; ++f) x[f] = (x[f] - V.mu[f]) * V.inv_sd[f];
            }
        }
        float y, dydx[kMlpIn];
        ok &= tc_rows128(t, phase, V, x, y, dydx);
        if (valid) {
            const float e = V.e_scale * y + V.e_shift;
            float dE[kMlpIn];
#pragma unroll
            for (int f = 0; f < kMlpIn; ++f) dE[f] = V.e_scale * dydx[f] * V.inv_sd[f];
            PairAcc acc;
            acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
            mlp_grad_to_forces(g, fi, fj, dE, acc);
            scatter<ENERGY>(a, p.i, p.j, acc, e);
            if (ENERGY) eacc[kHBCross] += (double)e;
            if (audit_step && audit_pick(k, step, a.audit_mod)) surrogate_audit(a, P, p.pidx, g, fi, fj, e, acc);
        }
        ok = __syncthreads_and(ok) != 0;
        tc::fence_after();
    }
    reduce_energies<ENERGY>(a, eacc);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(t.tmem, 256);
    }
    if (!ok && tid == 0) atomicOr(&a.st_rw->flags, kStBarrierTimeout);
}

// --------------------------------------------------- drop-in: HOOMD full nlist
// Minimum image of a difference of HOOMD's FP64 positions: the image count from an FP32
// estimate (an integer; either choice at exactly half a box is a valid image), the shift
// applied in FP64 by one fused multiply-add, so the FP32 result is the rounded exact
// difference. FP64 division, which costs tens of FP64 operations on this GPU's reduced
// FP64 pipe, is avoided.
__device__ __forceinline__ float min_image_d(double d, double L, float invL)
{
    const float n = rintf((float)d * invL);
    return (float)fma(-(double)n, L, d);
}

// HOOMD's FP64 particle arrays converted once per call (a thread per particle), so the
// pair loop reads FP32 only: hi = (x, y, z high parts, type bits), lo = (x, y, z low
// parts, charge), q = the quaternion. Positions are double-float (hi + lo = the FP64
// value to ~1e-14 relative), differences taken with image_delta as in the engine.
struct HoomdConvertArgs {
    int N;
    const double4_32a* pos;
    const double4_32a* quat;
    const double* charge;  // may be null: unit charges
    float4* hi;
    float4* lo;
    float4* q;
};

#ifndef OXG_DEVICE_FUNCTIONS_ONLY
__global__ void k_hoomd_convert(HoomdConvertArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const double4_32a p = a.pos[i];
    const double4_32a qd = a.quat[i];
    const float hx = (float)p.x, hy = (float)p.y, hz = (float)p.z;
    const int t = (int)(__double_as_longlong(p.w) & 0xffffffffLL);
    a.hi[i] = make_float4(hx, hy, hz, __int_as_float(t));
    a.lo[i] = make_float4((float)(p.x - (double)hx), (float)(p.y - (double)hy), (float)(p.z - (double)hz),
                          a.charge ? (float)a.charge[i] : 1.f);
    a.q[i] = make_float4((float)qd.x, (float)qd.y, (float)qd.z, (float)qd.w);
}
#endif

struct HoomdPairArgs {
    const unsigned char* params;
    int param_bytes;
    uint32_t mask;
    int N;
    const float4* hi;  // k_hoomd_convert's arrays
    const float4* lo;
    const float4* q;
    const uint32_t* n_neigh;
    const uint32_t* nlist;
    const unsigned long long* head_list;
    float3 Lf, invL;
    float4* force;
    float4* torque;
    float* virial;  // 6 * N, component-major pitch N (may be null)
    double* energy; // kNTerms (may be null)
    uint32_t* status;
};

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_pairs_hoomd(HoomdPairArgs a)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.N) return;  // whole warp exits together
    const float4 hi_i = a.hi[i], lo_i = a.lo[i];
    const float4 qi = a.q[i];
    const int ti = __float_as_int(hi_i.w);
    const int n_types = P.h().n_types;
    const float ci = lo_i.w;
    const int nn = (int)a.n_neigh[i];
    const unsigned long long head = a.head_list[i];
    float3 f = mk3(0.f, 0.f, 0.f), tq = mk3(0.f, 0.f, 0.f);
    float e_half = 0.f;
    float vir[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double eacc[kNTerms] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    bool bad = false;
    for (int k = lane; k < nn; k += 32) {
        const uint32_t j = a.nlist[head + k];
        if (j >= (uint32_t)a.N) {
            bad = true;
            continue;
        }
        const float4 hi_j = a.hi[j], lo_j = a.lo[j];
        const float3 dr = image_delta(hi_i, lo_i, hi_j, lo_j, a.Lf, a.invL);
        const float rsq = dot(dr, dr);
        const float4 qj = a.q[j];
        const int tj = __float_as_int(hi_j.w);
        if ((unsigned)ti >= (unsigned)n_types || (unsigned)tj >= (unsigned)n_types) {
            bad = true;
            continue;
        }
        const float cj = lo_j.w;
        PairAcc acc;
        acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
        float E[kNTerms] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (!eval_pair(P, a.mask, ti * kMaxTypes + tj, dr, rsq, qi, qj, ci, cj, acc, E)) continue;
        f += acc.fi;
        tq += acc.ti;
        if (ENERGY) {
#pragma unroll
            for (int t = 0; t < kNTerms; ++t) {
                eacc[t] += 0.5 * (double)E[t];
                e_half += 0.5f * E[t];
            }
        }
        if (a.virial) {  // HOOMD pair virial: 0.5 * dr (x) F_i
            vir[0] += 0.5f * dr.x * acc.fi.x;
            vir[1] += 0.5f * dr.x * acc.fi.y;
            vir[2] += 0.5f * dr.x * acc.fi.z;
            vir[3] += 0.5f * dr.y * acc.fi.y;
            vir[4] += 0.5f * dr.y * acc.fi.z;
            vir[5] += 0.5f * dr.z * acc.fi.z;
        }
    }
    f.x = warp_sum(f.x);
    f.y = warp_sum(f.y);
    f.z = warp_sum(f.z);
    tq.x = warp_sum(tq.x);
    tq.y = warp_sum(tq.y);
    tq.z = warp_sum(tq.z);
    if (ENERGY) e_half = warp_sum(e_half);
    if (a.virial)
#pragma unroll
        for (int c = 0; c < 6; ++c) vir[c] = warp_sum(vir[c]);
    if (lane == 0) {
        float4 F = a.force[i];
        F.x += f.x;
        F.y += f.y;
        F.z += f.z;
        F.w += e_half;
        a.force[i] = F;
        float4 T = a.torque[i];
        T.x += tq.x;
        T.y += tq.y;
        T.z += tq.z;
        a.torque[i] = T;
        if (a.virial)
            for (int c = 0; c < 6; ++c) a.virial[(size_t)c * a.N + i] += vir[c];
    }
    if (ENERGY && a.energy) {
#pragma unroll
        for (int t = 0; t < kNTerms; ++t) {
            const double s = warp_sum(eacc[t]);
            if (lane == 0 && s != 0.0) atomicAdd(a.energy + t, s);
        }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(a.status, kStBadIndex);
}

// ------------------------------------------------------------- drop-in: bonds
struct BondDropinArgs {
    const unsigned char* params;
    int param_bytes;
    int N, n_bonds;
    const double4_32a* pos;
    const double4_32a* quat;
    const int* bonds;  // 3 per bond
    double3 L;
    float3 invL;
    float4* force;
    float4* torque;
    float* virial;
    double* energy;    // 3 (fene, bexc, stack), may be null
    uint32_t* status;
};

#ifndef OXG_DEVICE_FUNCTIONS_ONLY  // the engine's translation unit defines the kernels
__global__ void __launch_bounds__(256) k_bonds_dropin(BondDropinArgs a)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    bool bad = false;
    if (b < a.n_bonds) {
        const int A = a.bonds[3 * b], B = a.bonds[3 * b + 1], bt = a.bonds[3 * b + 2];
        bad = A < 0 || B < 0 || A >= a.N || B >= a.N || bt < 0 || bt >= P.h().n_bond_types;
        double4_32a pA, pB;
        int tA = 0, tB = 0;
        if (!bad) {
            pA = a.pos[A];
            pB = a.pos[B];
            tA = (int)(__double_as_longlong(pA.w) & 0xffffffffLL);
            tB = (int)(__double_as_longlong(pB.w) & 0xffffffffLL);
            bad = (unsigned)tA >= (unsigned)P.h().n_types || (unsigned)tB >= (unsigned)P.h().n_types;
        }
        if (!bad) {
            const double dx = min_image_d(pB.x - pA.x, a.L.x, a.invL.x);
            const double dy = min_image_d(pB.y - pA.y, a.L.y, a.invL.y);
            const double dz = min_image_d(pB.z - pA.z, a.L.z, a.invL.z);
            BondAcc acc;
            bonded_pair(P.bonded(bt), make_double3(dx, dy, dz), a.quat[A], a.quat[B], tA, tB, acc);
            const float eh = (float)(0.5 * (acc.e[0] + acc.e[1] + acc.e[2]));
            atomicAdd(a.force + A, make_float4(-acc.fB.x, -acc.fB.y, -acc.fB.z, eh));
            atomicAdd(a.force + B, make_float4(acc.fB.x, acc.fB.y, acc.fB.z, eh));
            atomicAdd(a.torque + A, make_float4(acc.tA.x, acc.tA.y, acc.tA.z, 0.f));
            atomicAdd(a.torque + B, make_float4(acc.tB.x, acc.tB.y, acc.tB.z, 0.f));
            if (a.virial) {
                for (int c = 0; c < 6; ++c) {  // the half virial goes to both ends
                    atomicAdd(a.virial + (size_t)c * a.N + A, acc.vir[c]);
                    atomicAdd(a.virial + (size_t)c * a.N + B, acc.vir[c]);
                }
            }
            e0 = acc.e[0];
            e1 = acc.e[1];
            e2 = acc.e[2];
        }
    }
    if (a.energy) {
        e0 = warp_sum(e0);
        e1 = warp_sum(e1);
        e2 = warp_sum(e2);
        if ((threadIdx.x & 31) == 0) {
            if (e0 != 0.0) atomicAdd(a.energy + 0, e0);
            if (e1 != 0.0) atomicAdd(a.energy + 1, e1);
            if (e2 != 0.0) atomicAdd(a.energy + 2, e2);
        }
    }
    if (bad) atomicOr(a.status, kStBadIndex);
}
#endif

// ------------------------------------------------------------ neighbour list
struct NlistArgs {
    int N;
    const float4* pos;
    float4* pos_ref;
    const int4* excl;      // up to 4 bonded partners per particle (-1 = none)
    int3 nc;               // cells per dimension (>= 3 each when use_cells)
    int use_cells;
    int cell_cap;
    int n_cells;
    uint32_t* cell_count;  // 2 * n_cells (double-buffered by generation parity)
    int* cell_list;        // n_cells * cell_cap
    float3 L, invL;
    float rlist2, rshort2;
    int2* pairs_short;
    int2* pairs_long;
    int cap_short, cap_long;
    DevStatus* st;
};

__device__ __forceinline__ int cell_coord(float x, float invL, int n)
{
    float u = x * invL + 0.5f;
    u -= floorf(u);
    int c = (int)(u * (float)n);
    return c >= n ? n - 1 : (c < 0 ? 0 : c);
}

// Thread `t` of `nthreads`: zero the other parity's cell counts (for the next rebuild)
// and the pair counters.
__device__ __forceinline__ void nlist_zero_other(const NlistArgs& a, int t, int nthreads, uint32_t par)
{
    uint32_t* other = a.cell_count + (size_t)(par ^ 1u) * a.n_cells;
    for (int c = t; c < a.n_cells; c += nthreads) other[c] = 0u;
    if (t == 0) {
        a.st->n_short = 0u;
        a.st->n_long = 0u;
    }
}

// Bin particle i < N into the counts of generation parity `par`; record its position
// as the list's reference.
__device__ __forceinline__ void nlist_bin_particle(const NlistArgs& a, int i, uint32_t par)
{
    const float4 p = __ldcg(a.pos + i);
    a.pos_ref[i] = p;
    if (!a.use_cells) return;
    const int cx = cell_coord(p.x, a.invL.x, a.nc.x), cy = cell_coord(p.y, a.invL.y, a.nc.y),
              cz = cell_coord(p.z, a.invL.z, a.nc.z);
    const int c = (cz * a.nc.y + cy) * a.nc.x + cx;
    const uint32_t slot = atomicAdd(a.cell_count + (size_t)par * a.n_cells + c, 1u);
    if (slot < (uint32_t)a.cell_cap) a.cell_list[(size_t)c * a.cell_cap + slot] = i;
    else atomicOr(&a.st->flags, kStCellOverflow);
    atomicMax(&a.st->max_cell, slot + 1u);
}

#ifndef OXG_DEVICE_FUNCTIONS_ONLY
__global__ void k_nlist_bin(NlistArgs a)
{
    if (!a.st->rebuild) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t par = a.st->gen & 1u;
    nlist_zero_other(a, i, gridDim.x * blockDim.x, par);
    if (i < a.N) nlist_bin_particle(a, i, par);
}
#endif

__device__ __forceinline__ bool is_excluded(int4 e, int j) { return e.x == j || e.y == j || e.z == j || e.w == j; }

// Particle i's pairs j > i (bond-excluded, within r_list) from the cells of parity
// `par`, found by a whole warp (i warp-uniform): lanes 0..26 take the member counts of
// the 27 neighbour cells, a prefix sum flattens the candidates, and each round the 32
// lanes test 32 candidates at once (cell of a candidate by binary search over the
// prefix sums); found pairs are appended with one atomic per warp and list per round,
// or staged (below) when the warp handles many particles.
// Pairs found by a warp that handles many particles are staged in shared memory and
// appended to the global lists in batches: one counter atomic per batch instead of one
// per particle (100k particles: 200k same-address atomics per rebuild otherwise).
constexpr int kPairStage = 128;  // entries per list per warp
struct PairStage {
    int2* s;      // short-pair staging buffer (kPairStage entries, shared memory)
    int2* l;      // long-pair staging buffer
    int ns, nl;   // staged entries (warp-uniform)
};

// Append the warp's staged pairs of one list to the global list (all lanes).
__device__ __forceinline__ void stage_flush(const NlistArgs& a, int2* buf, int& n, uint32_t* counter,
                                            int2* list, int cap, bool& over)
{
    if (n == 0) return;
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, (uint32_t)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
        if (base + (uint32_t)k < (uint32_t)cap) list[base + k] = buf[k];
        else over = true;
    }
    __syncwarp();
    n = 0;
}

__device__ __forceinline__ void stage_flush_all(const NlistArgs& a, PairStage& sg)
{
    bool over = false;
    stage_flush(a, sg.s, sg.ns, &a.st->n_short, a.pairs_short, a.cap_short, over);
    stage_flush(a, sg.l, sg.nl, &a.st->n_long, a.pairs_long, a.cap_long, over);
    if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(&a.st->flags, kStPairOverflow);
}

__device__ __forceinline__ void nlist_pairs_warp(const NlistArgs& a, int i, uint32_t par,
                                                 PairStage* sg = nullptr)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint32_t* counts = a.cell_count + (size_t)par * a.n_cells;
    const float4 p = __ldcg(a.pos + i);
    const int4 ex = a.excl[i];
    int n_l = 0, cbase = 0;
    if (a.use_cells) {
        if (lane < 27) {
            const int cx = cell_coord(p.x, a.invL.x, a.nc.x), cy = cell_coord(p.y, a.invL.y, a.nc.y),
                      cz = cell_coord(p.z, a.invL.z, a.nc.z);
            const int x = (cx + lane % 3 - 1 + a.nc.x) % a.nc.x;
            const int y = (cy + (lane / 3) % 3 - 1 + a.nc.y) % a.nc.y;
            const int z = (cz + lane / 9 - 1 + a.nc.z) % a.nc.z;
            const int c = (z * a.nc.y + y) * a.nc.x + x;
            n_l = min((int)__ldcg(counts + c), a.cell_cap);
            cbase = c * a.cell_cap;
        }
    } else if (lane == 0) {
        n_l = a.N - 1 - i;  // all j > i
    }
    int incl = n_l;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl_off = incl - n_l;
    bool over = false;
    for (int k0 = 0; k0 < total; k0 += 32) {
        const int k = k0 + lane;
        const int kk = min(k, total - 1);
        // largest lane l < 27 whose range starts at or before kk (a non-empty cell)
        int lo = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int cand = lo + step;
            const int e = __shfl_sync(0xffffffffu, excl_off, cand & 31);
            if (cand < 27 && e <= kk) lo = cand;
        }
        const int start = __shfl_sync(0xffffffffu, excl_off, lo);
        const int cb = __shfl_sync(0xffffffffu, cbase, lo);
        bool is_short = false, is_long = false;
        int j = -1;
        if (k < total) {
            j = a.use_cells ? __ldcg(a.cell_list + cb + (kk - start)) : i + 1 + kk;
            if (j > i && !is_excluded(ex, j)) {
                const float4 pj = __ldcg(a.pos + j);
                const float3 d = min_image(mk3(p.x - pj.x, p.y - pj.y, p.z - pj.z), a.L, a.invL);
                const float r2 = dot(d, d);
                if (r2 < a.rlist2) {
                    is_short = r2 < a.rshort2;
                    is_long = !is_short;
                }
            }
        }
        const unsigned ms = __ballot_sync(0xffffffffu, is_short), ml = __ballot_sync(0xffffffffu, is_long);
        if (sg) {
            if (sg->ns + __popc(ms) > kPairStage)
                stage_flush(a, sg->s, sg->ns, &a.st->n_short, a.pairs_short, a.cap_short, over);
            if (sg->nl + __popc(ml) > kPairStage)
                stage_flush(a, sg->l, sg->nl, &a.st->n_long, a.pairs_long, a.cap_long, over);
            if (is_short) sg->s[sg->ns + __popc(ms & lt_mask)] = make_int2(i, j);
            if (is_long) sg->l[sg->nl + __popc(ml & lt_mask)] = make_int2(i, j);
            sg->ns += __popc(ms);
            sg->nl += __popc(ml);
            __syncwarp();
            continue;
        }
        uint32_t bs = 0, bl = 0;
        if (lane == 0) {
            if (ms) bs = atomicAdd(&a.st->n_short, (uint32_t)__popc(ms));
            if (ml) bl = atomicAdd(&a.st->n_long, (uint32_t)__popc(ml));
        }
        bs = __shfl_sync(0xffffffffu, bs, 0);
        bl = __shfl_sync(0xffffffffu, bl, 0);
        if (is_short) {
            const uint32_t slot = bs + __popc(ms & lt_mask);
            if (slot < (uint32_t)a.cap_short) a.pairs_short[slot] = make_int2(i, j);
            else over = true;
        }
        if (is_long) {
            const uint32_t slot = bl + __popc(ml & lt_mask);
            if (slot < (uint32_t)a.cap_long) a.pairs_long[slot] = make_int2(i, j);
            else over = true;
        }
    }
    if (over) atomicOr(&a.st->flags, kStPairOverflow);
    if (i == 0 && lane == 0) atomicAdd(&a.st->builds, 1u);
}

#ifndef OXG_DEVICE_FUNCTIONS_ONLY
// One warp per particle (grid-stride over particles).
__global__ void k_nlist_pairs(NlistArgs a)
{
    if (!a.st->rebuild) return;
    const uint32_t par = a.st->gen & 1u;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = w; i < a.N; i += nw) nlist_pairs_warp(a, i, par);
}
#endif

// ------------------------------------------------------------------ integrator
__device__ __forceinline__ void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    // Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

struct IntegArgs {
    int N;
    float4* pos;       // x, y, z (high parts), type
    float4* pos_lo;    // low parts
    float4* quat;
    float4* vel;       // vx, vy, vz, mass
    float4* angmom;
    float4* accel;     // (F + F_bath) / m from the last step two
    float4* tnet;      // T + T_bath (lab) from the last step two
    const float4* pos_ref;
    float4* force;
    float4* torque;
    DevStatus* st;
    float3 L, invL;
    float dt, kT, gamma, gamma_r;
    float half_buf2;   // (buffer / 2)^2
    float3 inertia;
    uint32_t seed_lo, seed_hi;
};

__device__ __forceinline__ float4 qmul_vec(float4 q, float3 t)
{
    // q * (0, t) with q = (s, x, y, z) in (.x, .y, .z, .w)
    return make_float4(-(q.y * t.x + q.z * t.y + q.w * t.z), q.x * t.x + q.z * t.z - q.w * t.y,
                       q.x * t.y + q.w * t.x - q.y * t.z, q.x * t.z + q.y * t.y - q.z * t.x);
}
__device__ __forceinline__ float3 rot_conj(float4 q, float3 v)
{
    const float4 c = make_float4(q.x, -q.y, -q.z, -q.w);
    const Frame f = quat_frame(c);
    return f.a1 * v.x + f.a2 * v.y + f.a3 * v.z;
}
__device__ __forceinline__ float4 perm(int k, float4 a)
{
    if (k == 1) return make_float4(-a.y, a.x, a.w, -a.z);
    if (k == 2) return make_float4(-a.z, -a.w, a.x, a.y);
    return make_float4(-a.w, a.z, -a.y, a.x);
}
// q4I = 1 / (4 I) of the axis (a multiplication on the dependency chain, not a division)
__device__ __forceinline__ void free_rotor(int k, float h, float q4I, float4& p, float4& q)
{
    const float4 pq = perm(k, q);
    const float phi = (p.x * pq.x + p.y * pq.y + p.z * pq.z + p.w * pq.w) * q4I;
    float s, c;
    sincosf(h * phi, &s, &c);
    const float4 pp = perm(k, p);
    p = make_float4(c * p.x + s * pp.x, c * p.y + s * pp.y, c * p.z + s * pp.z, c * p.w + s * pp.w);
    q = make_float4(c * q.x + s * pq.x, c * q.y + s * pq.y, c * q.z + s * pq.z, c * q.w + s * pq.w);
}

// x_hi + x_lo += d for a double-float coordinate (Knuth's TwoSum, FP32 only), then
// wrap the high part into [-L/2, L/2); subtracting L there is exact (Sterbenz).
__device__ __forceinline__ void dd_advance(float& hi, float& lo, float d, float L)
{
    const float s = lo + d;
    const float t = hi + s;
    const float bp = t - hi;
    lo = (hi - (t - bp)) + (s - bp);
    hi = t;
    if (hi >= 0.5f * L) hi -= L;
    else if (hi < -0.5f * L) hi += L;
}

// Per-particle integrator state (positions double-float).
struct PState {
    float4 x, xl, v, q, p;  // x.w = type bits, v.w = mass
    float4 ref;             // position at the last list build (the engine's step one)
};

// Step one with acceleration ac and net lab torque tn: v += dt/2 a; x += dt v
// (double-float, wrapped into [-L/2, L/2)); p += dt q*(0, t_body); NO_SQUISH free rotor
// (axes 3, 2 at dt/2, 1 at dt, 2, 3 at dt/2); renormalise q. Returns false on a
// non-finite result.
__device__ __forceinline__ bool step_one_pure(PState& s, float4 ac, float4 tn, float dt, float3 L,
                                              float3 inertia)
{
    s.v.x += 0.5f * dt * ac.x;
    s.v.y += 0.5f * dt * ac.y;
    s.v.z += 0.5f * dt * ac.z;
    dd_advance(s.x.x, s.xl.x, dt * s.v.x, L.x);
    dd_advance(s.x.y, s.xl.y, dt * s.v.y, L.y);
    dd_advance(s.x.z, s.xl.z, dt * s.v.z, L.z);
    float4 q = s.q, p = s.p;
    const float3 tb = rot_conj(q, mk3(tn.x, tn.y, tn.z));
    const float4 dq = qmul_vec(q, tb);
    p.x += dt * dq.x;
    p.y += dt * dq.y;
    p.z += dt * dq.z;
    p.w += dt * dq.w;
    const float q4x = 0.25f / inertia.x, q4y = 0.25f / inertia.y, q4z = 0.25f / inertia.z;
    free_rotor(3, 0.5f * dt, q4z, p, q);
    free_rotor(2, 0.5f * dt, q4y, p, q);
    free_rotor(1, dt, q4x, p, q);
    free_rotor(2, 0.5f * dt, q4y, p, q);
    free_rotor(3, 0.5f * dt, q4z, p, q);
    const float nq = rsqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    s.q = make_float4(q.x * nq, q.y * nq, q.z * nq, q.w * nq);
    s.p = p;
    return isfinite(s.x.x) && isfinite(s.x.y) && isfinite(s.x.z) && isfinite(s.q.x);
}

// Step two (HOOMD TwoStepLangevin semantics) with force F and torque T: bath force
// u*sqrt(6 gamma kT/dt) - gamma v, u uniform in [-1, 1); bath torque (body frame)
// n*sqrt(2 gamma_r kT/dt) - gamma_r L/I, n standard normal; a = (F + F_bath)/m;
// v += dt/2 a; tnet = T + R(q) T_bath; p += dt q*(0, t_body). The Philox counter is
// (tag, step, stream) under the key (seed_lo, seed_hi).
// The Langevin bath noise of one particle and step: translational u * sqrt(6 gamma kT/dt)
// (u uniform in [-1, 1)) and rotational n * sqrt(2 gamma_r kT/dt) (n standard normal,
// Box-Muller). It depends on the tag, step and seed alone, so the run kernel computes it
// while it waits at the force barrier.
struct LangevinNoise {
    float3 t, r;
};
__device__ __forceinline__ LangevinNoise langevin_noise(uint32_t tag, unsigned long long step, uint32_t seed_lo,
                                                        uint32_t seed_hi, float dt, float kT, float gamma,
                                                        float gamma_r)
{
    uint32_t r0[4] = {tag, (uint32_t)step, (uint32_t)(step >> 32), 0u};
    uint32_t r1[4] = {tag, (uint32_t)step, (uint32_t)(step >> 32), 1u};
    philox4x32(r0, seed_lo, seed_hi);
    philox4x32(r1, seed_lo, seed_hi);
    const float ct = sqrtf(6.f * gamma * kT / dt);
    const float cr = sqrtf(2.f * gamma_r * kT / dt);
    const float inv31 = 1.f / 2147483648.f;
    LangevinNoise n;
    n.t = mk3((float)(int32_t)r0[0] * inv31 * ct, (float)(int32_t)r0[1] * inv31 * ct,
              (float)(int32_t)r0[2] * inv31 * ct);
    // Box-Muller on two word pairs
    const float u1 = ((float)r1[0] + 1.f) * 2.3283064365386963e-10f;
    const float u2 = (float)r1[1] * 2.3283064365386963e-10f;
    const float u3 = ((float)r1[2] + 1.f) * 2.3283064365386963e-10f;
    const float u4 = (float)r1[3] * 2.3283064365386963e-10f;
    const float ra = sqrtf(-2.f * logf(fminf(u1, 1.f))), rb = sqrtf(-2.f * logf(fminf(u3, 1.f)));
    float s2a, c2a, s2b, c2b;
    sincospif(2.f * u2, &s2a, &c2a);
    sincospif(2.f * u4, &s2b, &c2b);
    n.r = mk3(ra * c2a * cr, ra * s2a * cr, rb * c2b * cr);
    return n;
}

// Step two with the particle's bath noise n: a = (F + F_bath)/m with F_bath = n.t -
// gamma v; tnet = T + R(q) (n.r - gamma_r L/I); v += dt/2 a; p += dt q*(0, t_body).
__device__ __forceinline__ void step_two_noise(PState& s, float4 F, float4 T, const LangevinNoise& n, float dt,
                                               float gamma, float gamma_r, float3 inertia, float4& ac, float4& tn)
{
    const float minv = 1.f / s.v.w;
    ac.x = (F.x + n.t.x - gamma * s.v.x) * minv;
    ac.y = (F.y + n.t.y - gamma * s.v.y) * minv;
    ac.z = (F.z + n.t.z - gamma * s.v.z) * minv;
    ac.w = 0.f;
    const float4 q = s.q;
    float4 p = s.p;
    // s = (1/2 conj(q) p).v : body-frame angular momentum
    const float sx = 0.5f * (q.x * p.y - p.x * q.y - (q.z * p.w - q.w * p.z));
    const float sy = 0.5f * (q.x * p.z - p.x * q.z - (q.w * p.y - q.y * p.w));
    const float sz = 0.5f * (q.x * p.w - p.x * q.w - (q.y * p.z - q.z * p.y));
    const float3 bt = mk3(n.r.x - gamma_r * sx * (1.f / inertia.x), n.r.y - gamma_r * sy * (1.f / inertia.y),
                          n.r.z - gamma_r * sz * (1.f / inertia.z));
    const Frame fq = quat_frame(q);
    const float3 btl = fq.a1 * bt.x + fq.a2 * bt.y + fq.a3 * bt.z;
    tn = make_float4(T.x + btl.x, T.y + btl.y, T.z + btl.z, 0.f);
    s.v.x += 0.5f * dt * ac.x;
    s.v.y += 0.5f * dt * ac.y;
    s.v.z += 0.5f * dt * ac.z;
    const float3 tb = rot_conj(q, mk3(tn.x, tn.y, tn.z));
    const float4 dq = qmul_vec(q, tb);
    p.x += dt * dq.x;
    p.y += dt * dq.y;
    p.z += dt * dq.z;
    p.w += dt * dq.w;
    s.p = p;
}

__device__ __forceinline__ void step_two_pure(PState& s, float4 F, float4 T, uint32_t tag,
                                              unsigned long long step, uint32_t seed_lo,
                                              uint32_t seed_hi, float dt, float kT, float gamma,
                                              float gamma_r, float3 inertia, float4& ac, float4& tn)
{
    const LangevinNoise n = langevin_noise(tag, step, seed_lo, seed_hi, dt, kT, gamma, gamma_r);
    step_two_noise(s, F, T, n, dt, gamma, gamma_r, inertia, ac, tn);
}

__device__ __forceinline__ PState load_pstate(const IntegArgs& a, int i)
{
    PState s;
    s.x = a.pos[i];
    s.xl = a.pos_lo[i];
    s.v = a.vel[i];
    s.q = a.quat[i];
    s.p = a.angmom[i];
    s.ref = a.pos_ref[i];  // with the state loads: after the stores it would wait a round trip
    return s;
}

// Step one of particle i in the resident arrays; zeroes its force accumulators and
// reports whether it moved more than half the buffer since the last list build.
__device__ __forceinline__ void particle_step_one(const IntegArgs& a, int i, PState s, float4 ac,
                                                  float4 tn, bool& far, bool& bad)
{
    bad = !step_one_pure(s, ac, tn, a.dt, a.L, a.inertia);
    a.pos[i] = s.x;
    a.pos_lo[i] = s.xl;
    a.vel[i] = s.v;
    a.quat[i] = s.q;
    a.angmom[i] = s.p;
    a.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    a.torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 r = s.ref;
    const float3 d = min_image(mk3(s.x.x - r.x, s.x.y - r.y, s.x.z - r.z), a.L, a.invL);
    far = dot(d, d) > a.half_buf2;
}

__device__ __forceinline__ void particle_step_two(const IntegArgs& a, int i,
                                                  unsigned long long step, PState& s, float4& ac,
                                                  float4& tn)
{
    step_two_pure(s, __ldcg(a.force + i), __ldcg(a.torque + i), (uint32_t)i, step, a.seed_lo, a.seed_hi, a.dt, a.kT,
                  a.gamma, a.gamma_r, a.inertia, ac, tn);
}

// First step one of a run (accelerations and torques from prepRun / the last step).
__device__ __forceinline__ void reset_queues(DevStatus* st)
{
    if (blockIdx.x == 0 && threadIdx.x < kNQ) st->qcount[threadIdx.x] = 0u;
}

#ifndef OXG_DEVICE_FUNCTIONS_ONLY
__global__ void k_step_one(IntegArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    reset_queues(a.st);
    bool far = false, bad = false;
    if (i < a.N) particle_step_one(a, i, load_pstate(a, i), a.accel[i], a.tnet[i], far, bad);
    if (__syncthreads_or(far) && threadIdx.x == 0) atomicOr(&a.st->rebuild, 1u);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&a.st->flags, kStNonFinite);
}

// Last step two of a run: also stores a and tnet so a later run can continue.
__global__ void k_step_two(IntegArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    reset_queues(a.st);
    if (i >= a.N) return;
    PState s = load_pstate(a, i);
    float4 ac, tn;
    particle_step_two(a, i, a.st->step, s, ac, tn);
    a.vel[i] = s.v;
    a.angmom[i] = s.p;
    a.accel[i] = ac;
    a.tnet[i] = tn;
}

// Step two of step n fused with step one of step n + 1 (per particle, no grid-wide
// dependency between them): the bath forces, kicks and drift in one pass.
__global__ void k_step_two_one(IntegArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    reset_queues(a.st);
    bool far = false, bad = false;
    if (i < a.N) {
        PState s = load_pstate(a, i);
        float4 ac, tn;
        particle_step_two(a, i, a.st->step, s, ac, tn);
        particle_step_one(a, i, s, ac, tn, far, bad);
    }
    if (__syncthreads_or(far) && threadIdx.x == 0) atomicOr(&a.st->rebuild, 1u);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&a.st->flags, kStNonFinite);
}

// Start (or replay) of a run on the device: the RNG step counter, cleared flags, a
// forced neighbour-list rebuild and empty queues (no host-to-device copies needed).
__global__ void k_begin_run(DevStatus* st, unsigned long long step, uint32_t rebuild)
{
    if (threadIdx.x == 0) {
        st->step = step;
        st->flags = 0u;
        st->rebuild = rebuild;
        st->qspill = 0u;
        st->rb[0] = 0u;
        st->rb[1] = 0u;
    }
    if (threadIdx.x < kNQ) st->qcount[threadIdx.x] = 0u;
}

// Flags a neighbour-list rebuild if a particle is more than half the buffer away from
// its position at the last build.
__global__ void k_check_moved(IntegArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < a.N) {
        const float4 x = a.pos[i], r = a.pos_ref[i];
        const float3 d = min_image(mk3(x.x - r.x, x.y - r.y, x.z - r.z), a.L, a.invL);
        far = !(dot(d, d) <= a.half_buf2);
    }
    if (__syncthreads_or(far) && threadIdx.x == 0) atomicOr(&a.st->rebuild, 1u);
}

// prepRun: accelerations from the forces alone (no bath), as HOOMD does at run start.
__global__ void k_prep_accel(IntegArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    reset_queues(a.st);
    if (i >= a.N) return;
    const float4 F = a.force[i], T = a.torque[i], v = a.vel[i];
    const float minv = 1.f / v.w;
    a.accel[i] = make_float4(F.x * minv, F.y * minv, F.z * minv, 0.f);
    a.tnet[i] = make_float4(T.x, T.y, T.z, 0.f);
}
#endif

// ------------------------------------------------------- persistent run kernel
// One cooperative launch runs many MD step bodies; its blocks (all co-resident, which
// the cooperative launch guarantees) meet at grid barriers between the phases, so the
// code stays in the instruction caches and the parameters in shared memory for the
// whole launch instead of being fetched again by five launches per step.
#ifndef OXG_RUN_THREADS
#define OXG_RUN_THREADS 256
#endif
#ifndef OXG_RUN_BLOCKS_PER_SM
#define OXG_RUN_BLOCKS_PER_SM (512 / OXG_RUN_THREADS)
#endif
// The parameters of one run of the run kernel: from the launch's arguments for its first
// run, from the host's request for each further run of a host session (below).
struct RunCmd {
    int bodies;                // step bodies of the run
    int closing;               // the last body is the run's last step (step two only)
    int prologue;              // run start kind (RunArgs::prologue)
    int reuse_ok;              // kind 3: the force arrays hold the device state's forces
    uint32_t rebuild0;         // the lists are new: rebuild whatever the displacements
    uint32_t seq;              // stored last into the status mirror at the run's end
    unsigned long long step0;  // the system's timestep at the run's start (RNG counter)
    const float4* hin[5];      // host state read at the run start (mapped), or null
    float4* hout[5];           // host arrays written by the closing body (mapped), or null
};

// A host session (oxg_system_set_host_session): the run kernel stays resident after a
// host-state run and serves the host's next requests, each a run of the same kind, until
// the host asks it to leave or no request comes within the idle time. The host writes a
// request into page-locked memory, its sequence number last; block 0 of the kernel polls
// that word (bounded by the idle time), copies the request into the barrier's command
// and the blocks meet at a grid barrier before the run.
struct HostRequest {
    uint32_t seq;              // stored last by the host: a request differs from the last one
    uint32_t quit;             // leave the kernel instead of running
    int bodies;
    int reuse_ok;
    unsigned long long step0;
    const float4* hin[5];      // device aliases of the caller's page-locked arrays
    float4* hout[5];
};

struct GridBarrier {
    uint32_t arrive;  // bit 31 flips each time every block has arrived
    uint32_t abort;   // set by a block whose wait gave up: the others leave too
    uint32_t exits;   // blocks that have left the launch (the last one resets it)
    uint32_t pad[29]; // a line of its own
    uint32_t go;      // host session: the next command is a run (0: leave)
    uint32_t pad2;
    RunCmd cmd;       // host session: the next run, written by block 0 before a grid barrier
    HostRequest req;  // host session: block 0's copy of the host's request
};
static_assert(sizeof(HostRequest) % sizeof(unsigned long long) == 0 && sizeof(HostRequest) <= 32 * 8,
              "a host request is copied one 8-byte word per lane of a warp");
static_assert(sizeof(RunCmd) % sizeof(unsigned long long) == 0, "a run command is copied in 8-byte words");

constexpr long long kBarrierSpinLimit = 1LL << 22;  // polls of an L2 round trip: ~1 s on a GB300 (0.23 us a poll)
constexpr long long kServeSpinLimit = 1LL << 30;    // polls of a host request (the idle time ends it first)

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}


__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Arrive at the grid barrier (the whole block); the returned token (thread 0) is the
// counter before this block's arrival. Work that does not depend on the other blocks
// may run between grid_arrive and grid_wait.
__device__ __forceinline__ uint32_t grid_arrive(GridBarrier* gb)
{
    __syncthreads();
    uint32_t old = 0u;
    if (threadIdx.x == 0) {
        const uint32_t add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(&gb->arrive), "r"(add) : "memory");
    }
    return old;
}

// Wait until every block has arrived (bit 31 of the counter differs from the token's).
// Returns false if the wait gave up (after kBarrierSpinLimit polls) or another block
// did; the caller must then return.
__device__ __forceinline__ bool grid_wait(GridBarrier* gb, uint32_t old)
{
    __shared__ int bar_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        long long polls = 0;
        while (((old ^ ld_acquire(&gb->arrive)) & 0x80000000u) == 0u) {
            if ((++polls & 63) == 0) {  // the abort word and the limit every 64 polls
                if (ld_volatile(&gb->abort)) {
                    ok = 0;
                    break;
                }
                if (polls > kBarrierSpinLimit) {
                    atomicExch(&gb->abort, 1u);
                    ok = 0;
                    break;
                }
            }
        }
        bar_ok = ok;
    }
    __syncthreads();
    return bar_ok != 0;
}

// Arrive-and-wait over all blocks of the launch. Block 0 adds 2^31 - (blocks - 1),
// every other block 1, so bit 31 of the counter flips exactly when the last block
// arrives (and the counter needs no reset). The arrival is a release and the polls are
// acquires (after the block's __syncthreads), so every write before the barrier is
// visible to every read after it.
__device__ __forceinline__ bool grid_barrier(GridBarrier* gb)
{
    return grid_wait(gb, grid_arrive(gb));
}

struct RunArgs {
    ForceArgs f;
    NlistArgs n;
    IntegArgs g;
    GridBarrier* bar;
    int bodies;   // step bodies in this launch
    int closing;  // the last body is the run's last step (step two only)
    unsigned long long step0;  // the system's timestep at the launch (RNG counter), every launch
    // run start in the same launch (the first launch of a run() call): 0 none, 1 full
    // (list check, forces of the current state), 2 with the forces of the last step (the
    // state has not changed since a run ended: the force arrays hold its final forces),
    // 3 from host state (hin): kind 2 if it equals the device state and reuse_ok, else 1
    int prologue;
    uint32_t rebuild0;         // the lists are new: rebuild whatever the displacements
    float4* ck[5];             // checkpoint of pos, pos_lo, quat, vel, angmom for a replay
    // host-state runs (the k_run<true> instantiation): mapped page-locked host arrays of
    // pos, pos_lo, quat, vel, angmom read at the run start (hin) and written by the run's
    // closing body (hout); null when not used by this launch
    const float4* hin[5];
    float4* hout[5];
    int reuse_ok;              // kind 3: the force arrays hold the device state's forces
    DevStatus* st_mirror;      // host-mapped copy of the status written by the last block
                               // to leave (null: the host copies the status itself)
    uint32_t seq;              // this launch's sequence number, stored last into st_mirror->seq
    // host session (k_run<true> only): after each run, wait up to idle_ns for the next
    // request in req (mapped host memory); null: leave after the launch's run
    const HostRequest* req;
    unsigned long long idle_ns;
};



// L2 prefetch of `bytes` from p, one 128-byte line per thread in turn (fire and forget).
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes, int tid, int nthreads)
{
    const char* c = static_cast<const char*>(p);
    for (size_t off = (size_t)tid * 128; off < bytes; off += (size_t)nthreads * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(c + off));
}

#ifndef OXG_DEVICE_FUNCTIONS_ONLY
// Each body: [neighbour-list rebuild if flagged: bin | pairs] | forces: each block's
// phase A, then (a block barrier) its phase B on the pairs it queued and its slice of
// the bonds [| pairs that did not fit a block's queues, by every block] | step two +
// step one of the next step. Grid barriers separate the brackets. A body's rebuild
// request is read by every block before the force barrier and cleared after it (the
// requests alternate between two words by body parity); a list overflow ends the
// launch (the host grows the lists and replays from its checkpoint).
//
// The first launch of a run() call starts with the run start as body -1 (HOOMD's
// prepRun): reset the step counter, flags and queues, checkpoint the state for a
// replay, clear the accumulators and check the displacements since the last list
// build | [rebuild if the lists are new or a particle moved half the buffer] | forces
// of the current state, no step advance | a = F/m and step one of the first step.
constexpr int kRunThreads = OXG_RUN_THREADS;  // threads per block of the run kernel
constexpr int kBondStage = 512;               // bonds a block stages in shared memory
template <bool HOST_IO>
__global__ void __launch_bounds__(kRunThreads, OXG_RUN_BLOCKS_PER_SM) k_run(RunArgs a)
{
    const ParamView P = stage_params(a.f.params, a.f.param_bytes);
    DevStatus* st = a.f.st_rw;
    const int lane = threadIdx.x & 31;
    const int gwarp = spread_warp();
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int gthread = gwarp * 32 + lane, nthreads = nwarps * 32;
    double eacc[kNTerms + 3];  // unused: MD steps evaluate no energies
    bool bad_type = false;
    // the stored pair counts and this thread's first short- and long-pair entries, read
    // at the launch's start (issued here, they arrive while the run start works) and
    // again after each list build (they change only there)
    int ns_known, nl_known;
    int2 first_pair[2];
    auto load_known = [&]() {
        ns_known = (int)min(ld_volatile(&st->n_short), (uint32_t)a.f.cap_short);
        nl_known = (int)min(ld_volatile(&st->n_long), (uint32_t)a.f.cap_long);
        first_pair[0] = gwarp * 32 + lane < ns_known ? __ldcg(a.f.pairs_short + gwarp * 32 + lane) : make_int2(0, 0);
        int v0, vstride;
        long_units(gwarp, nwarps, ns_known, nl_known, v0, vstride);
        first_pair[1] = (v0 >= 0 && v0 * 32 + lane < nl_known) ? __ldcg(a.f.pairs_long + v0 * 32 + lane)
                                                               : make_int2(0, 0);
    };
    load_known();
    // the block's slice of the (constant) bond table, staged once per launch when it fits
    __shared__ int4 bond_stage[kBondStage];
    const int4* bonds_here = nullptr;
    {
        const int nb = a.f.bonded ? a.f.n_bonds : 0;
        const int bb0 = (int)((long long)nb * blockIdx.x / gridDim.x);
        const int bb1 = (int)((long long)nb * (blockIdx.x + 1) / gridDim.x);
        if (bb1 - bb0 <= kBondStage) {
            for (int k = threadIdx.x; k < bb1 - bb0; k += blockDim.x) bond_stage[k] = a.f.bonds[bb0 + k];
            bonds_here = bond_stage;  // read after phase A's first block barrier
        }
    }
    // this run's parameters: the launch's; in a host session, each further request's
    __shared__ RunCmd cmd;
    __shared__ uint32_t serve_go;
    if (threadIdx.x == 0) {
        cmd.bodies = a.bodies;
        cmd.closing = a.closing;
        cmd.prologue = a.prologue;
        cmd.reuse_ok = a.reuse_ok;
        cmd.rebuild0 = a.rebuild0;
        cmd.seq = a.seq;
        cmd.step0 = a.step0;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            cmd.hin[k] = a.hin[k];
            cmd.hout[k] = a.hout[k];
        }
    }
    __syncthreads();
    for (;;) {  // one run per pass
        bool spec_used = false;  // the run start took the first step one in its own pass
        uint32_t spec_rebuild = 0u;  // then: body 0's rebuild request, read by the run start
        bool completed = false;  // the run's last body ran to its end
        bad_type = false;
        // the RNG step of body b is step0 + b + 1 (block 0 advances st->step to match); the
        // host passes step0 to every run: reading st->step here would race with block 0's
        // first increment in a block that starts late
        const unsigned long long step_base = cmd.step0;
        for (int body = cmd.prologue ? -1 : 0; body < cmd.bodies; ++body) {
            const bool pro = body < 0;
            bool reuse = pro && cmd.prologue == 2;  // the last step's forces are this state's
            bool rebuild;
            if (pro) {
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    st->step = cmd.step0;
                    st->flags = 0u;
                    st->rebuild = 0u;
                    st->qspill = 0u;
                    st->rb[0] = 0u;
                    st->rb[1] = 0u;
                }
                if (blockIdx.x == 0 && threadIdx.x < kNQ) st->qcount[threadIdx.x] = 0u;
                const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                const bool from_host = HOST_IO && cmd.prologue == 3;
                // When the force arrays may hold this state's forces (kind 2; kind 3 with
                // reuse_ok, which is only known once every block has compared its particles),
                // this pass also takes the first step's step one (a = F/m from those forces),
                // saving the run start's own step pass and its grid barrier. If the host state
                // turns out to differ, the pass after the barrier restores the state from the
                // checkpoint and the run start continues as kind 1 does.
                const bool spec = cmd.prologue == 2 || (from_host && cmd.reuse_ok != 0);
                bool far = false, diff = false, sfar = false, sbad = false;
                {
                    // the first body's reads into L2 while the run start works (after an idle
                    // period L2 may hold none of them): pair lists, bonds, charges
                    prefetch_l2(a.f.pairs_short, (size_t)ns_known * sizeof(int2), gthread, nthreads);
                    prefetch_l2(a.f.pairs_long, (size_t)nl_known * sizeof(int2), gthread, nthreads);
                    if (a.f.bonded) prefetch_l2(a.f.bonds, (size_t)a.f.n_bonds * sizeof(int4), gthread, nthreads);
                    if (a.f.charge) prefetch_l2(a.f.charge, (size_t)a.g.N * sizeof(float), gthread, nthreads);
                }
                for (int i = gthread; i < a.g.N; i += nthreads) {
                    float4 v[5], F = zero, T = zero, r;
                    if (from_host) {
                        // the host's state (mapped memory) into the device arrays; compared
                        // bit for bit with what they held
                        // every load issued before any store: a store to a device array
                        // could alias a later host load for the compiler, which would then
                        // serialise the five host round trips
                        float4* const dv[5] = {a.g.pos, a.g.pos_lo, a.g.quat, a.g.vel, a.g.angmom};
                        float4 o[5];
#pragma unroll
                        for (int k = 0; k < 5; ++k) v[k] = cmd.hin[k][i];
#pragma unroll
                        for (int k = 0; k < 5; ++k) o[k] = dv[k][i];
                        r = a.g.pos_ref[i];
                        if (spec) {
                            F = __ldcg(a.g.force + i);
                            T = __ldcg(a.g.torque + i);
                        }
                        if ((unsigned)__float_as_int(v[0].w) >= (unsigned)P.h().n_types)
                            bad_type = true;  // reported after the run (the kernels skip the particle)
#pragma unroll
                        for (int k = 0; k < 5; ++k) {
                            diff |= __float_as_uint(v[k].x) != __float_as_uint(o[k].x) ||
                                    __float_as_uint(v[k].y) != __float_as_uint(o[k].y) ||
                                    __float_as_uint(v[k].z) != __float_as_uint(o[k].z) ||
                                    __float_as_uint(v[k].w) != __float_as_uint(o[k].w);
                            dv[k][i] = v[k];
                        }
                    } else {
                        v[0] = a.g.pos[i];
                        v[1] = a.g.pos_lo[i];
                        v[2] = a.g.quat[i];
                        v[3] = a.g.vel[i];
                        v[4] = a.g.angmom[i];
                        r = a.g.pos_ref[i];
                        if (spec) {
                            F = __ldcg(a.g.force + i);
                            T = __ldcg(a.g.torque + i);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 5; ++k) a.ck[k][i] = v[k];
                    if (!spec && reuse) continue;  // forces kept; the lists are valid for this state
                    if (!from_host && !spec) {     // (from host state: zeroed below once it is known to differ)
                        a.g.force[i] = zero;
                        a.g.torque[i] = zero;
                    }
                    if (!reuse) {  // the state's own displacement since the last list build
                        const float3 d = min_image(mk3(v[0].x - r.x, v[0].y - r.y, v[0].z - r.z), a.g.L, a.g.invL);
                        far |= !(dot(d, d) <= a.g.half_buf2);
                    }
                    if (spec) {
                        // the first step one (writes the stepped state, zeroes the accumulators)
                        PState ps;
                        ps.x = v[0];
                        ps.xl = v[1];
                        ps.q = v[2];
                        ps.v = v[3];
                        ps.p = v[4];
                        ps.ref = r;
                        const float minv = 1.f / ps.v.w;
                        bool f1 = false, b1 = false;
                        particle_step_one(a.g, i, ps, make_float4(F.x * minv, F.y * minv, F.z * minv, 0.f),
                                          make_float4(T.x, T.y, T.z, 0.f), f1, b1);
                        sfar |= f1;
                        sbad |= b1;
                    }
                }
                if (spec && __syncthreads_or(sfar) && threadIdx.x == 0) atomicOr(&st->spec_far, 1u);
                if (__syncthreads_or(far) && threadIdx.x == 0) atomicOr(&st->moved, 1u);
                if (from_host && __syncthreads_or(diff) && threadIdx.x == 0) atomicOr(&st->changed, 1u);
                if (!grid_barrier(a.bar)) break;  // the counters above are reset for every block
                // the words the run start's pass left, read together (one L2 round trip, not
                // one after another): whether the host state differed, the first step one's
                // displacement test and the rebuild request body 0 would read (nothing writes
                // either of the last two between this barrier and body 0's force barrier)
                const uint32_t v_changed = from_host ? ld_volatile(&st->changed) : 0u;
                const uint32_t v_sfar = spec ? ld_volatile(&st->spec_far) : 0u;
                const uint32_t v_rebuild = spec ? ld_volatile(&st->rebuild) : 0u;
                if (from_host) {
                    reuse = cmd.reuse_ok != 0 && v_changed == 0u;  // the same in every block
                    if (!reuse) {
                        for (int i = gthread; i < a.g.N; i += nthreads) {
                            if (spec) {  // undo the first step one: the state from the checkpoint
                                a.g.pos[i] = a.ck[0][i];
                                a.g.pos_lo[i] = a.ck[1][i];
                                a.g.quat[i] = a.ck[2][i];
                                a.g.vel[i] = a.ck[3][i];
                                a.g.angmom[i] = a.ck[4][i];
                            }
                            a.g.force[i] = zero;
                            a.g.torque[i] = zero;
                        }
                        if (!grid_barrier(a.bar)) break;  // zeroed before any block scatters forces
                    }
                }
                if (spec && reuse) {
                    // the first step one is done: its forces (body 0) come next; body 0
                    // takes its rebuild request from the words read above
                    if (__syncthreads_or(sbad) && threadIdx.x == 0) atomicOr(&st->flags, kStNonFinite);
                    spec_used = true;
                    spec_rebuild = v_rebuild | v_sfar;
                    continue;
                }
                rebuild = !reuse && (cmd.rebuild0 != 0u || ld_volatile(&st->moved) != 0u);
            } else {
                // rebuild requests: body 0 reads the one left by the run start or the previous
                // launch, body b > 0 the one the step phase of body b - 1 left in rb[b & 1]
                if (body == 0 && spec_used) rebuild = spec_rebuild != 0u;
                else rebuild = ld_volatile(body == 0 ? &st->rebuild : &st->rb[body & 1]) != 0u;
            }
            if (rebuild) {
                const uint32_t par = ld_volatile(&st->gen) & 1u;
                nlist_zero_other(a.n, gthread, nthreads, par);
                for (int i = gthread; i < a.n.N; i += nthreads) nlist_bin_particle(a.n, i, par);
                if (!grid_barrier(a.bar)) break;
                {
                    __shared__ int2 stage_buf[2][kRunThreads / 32][kPairStage];
                    PairStage sg{stage_buf[0][threadIdx.x >> 5], stage_buf[1][threadIdx.x >> 5], 0, 0};
                    for (int i = gwarp; i < a.n.N; i += nwarps) nlist_pairs_warp(a.n, i, par, &sg);
                    stage_flush_all(a.n, sg);
                }
                if (!grid_barrier(a.bar)) break;
                if (ld_volatile(&st->flags) & (kStCellOverflow | kStPairOverflow)) break;
            }
            if (rebuild) load_known();
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                if (rebuild) st->gen += 1u;
                if (!pro) st->step += 1ull;
            }
            // this thread's first particle's bath noise for step two, computed between its
            // block's arrival at the force barrier and the barrier's release
            const unsigned long long step = step_base + (unsigned long long)(body + 1);
            LangevinNoise nz;
            const bool have_nz = !pro && gthread < a.g.N;
            if (!reuse) {
                // phase B on the block's own queues: a block barrier, not a grid barrier
                forces_a_body<false, true>(a.f, P, gwarp, nwarps, eacc, bad_type, ns_known, nl_known, first_pair);
                forces_b_local<false>(a.f, P, eacc, bad_type, bonds_here);
                const uint32_t tok = grid_arrive(a.bar);
                if (have_nz)
                    nz = langevin_noise((uint32_t)gthread, step, a.g.seed_lo, a.g.seed_hi, a.g.dt, a.g.kT, a.g.gamma,
                                        a.g.gamma_r);
                if (!grid_wait(a.bar, tok)) break;
                if (ld_volatile(&st->qspill)) {  // pairs that did not fit a block's queues
                    forces_b_body<false, false>(a.f, P, gwarp, nwarps, eacc, bad_type);
                    if (!grid_barrier(a.bar)) break;
                    if (blockIdx.x == 0 && threadIdx.x == 0) st->qspill = 0u;  // read a barrier ago
                }
            }
            // every block read this body's rebuild request before the last barrier
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                if (body == 0) {
                    st->rebuild = 0u;
                    st->spec_far = 0u;
                    if (spec_used) {  // the run start's step pass, which clears these, was skipped
                        st->moved = 0u;
                        st->changed = 0u;
                    }
                } else if (body > 0) {
                    st->rb[body & 1] = 0u;
                }
            }
            // step two of this step (+ step one of the next); at run start a = F/m and
            // step one of the first step
            const bool last = cmd.closing && body == cmd.bodies - 1;
            if (blockIdx.x == 0) {
                if (threadIdx.x < kNQ) st->qcount[threadIdx.x] = 0u;
                if (pro && threadIdx.x == 32) st->moved = 0u;    // read two barriers ago
                if (pro && threadIdx.x == 64) st->changed = 0u;  // read two barriers ago
            }
            bool far = false, bad = false;
            for (int i = gthread; i < a.g.N; i += nthreads) {
                PState s = load_pstate(a.g, i);
                float4 ac, tn;
                if (pro) {
                    const float4 F = __ldcg(a.g.force + i), T = __ldcg(a.g.torque + i);
                    const float minv = 1.f / s.v.w;
                    ac = make_float4(F.x * minv, F.y * minv, F.z * minv, 0.f);
                    tn = make_float4(T.x, T.y, T.z, 0.f);
                } else if (have_nz && i == gthread) {
                    step_two_noise(s, __ldcg(a.g.force + i), __ldcg(a.g.torque + i), nz, a.g.dt, a.g.gamma,
                                   a.g.gamma_r, a.g.inertia, ac, tn);
                } else {
                    particle_step_two(a.g, i, step, s, ac, tn);
                }
                if (last) {
                    a.g.vel[i] = s.v;
                    a.g.angmom[i] = s.p;
                    a.g.accel[i] = ac;
                    a.g.tnet[i] = tn;
                    if (HOST_IO && cmd.hout[0]) {  // the run's final state to the host (mapped)
                        cmd.hout[0][i] = s.x;
                        cmd.hout[1][i] = s.xl;
                        cmd.hout[2][i] = s.q;
                        cmd.hout[3][i] = s.v;
                        cmd.hout[4][i] = s.p;
                    }
                } else {
                    bool f1 = false, b1 = false;
                    particle_step_one(a.g, i, s, ac, tn, f1, b1);
                    far |= f1;
                    bad |= b1;
                }
            }
            // the next body's rebuild request: the run start's to st->rebuild (read by body 0),
            // body b's to rb[(b + 1) & 1] (cleared by body b - 1 after its force barrier)
            if (__syncthreads_or(far) && threadIdx.x == 0) atomicOr(pro ? &st->rebuild : &st->rb[(body + 1) & 1], 1u);
            if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&st->flags, kStNonFinite);
            if (body == cmd.bodies - 1) {  // the launch's last body: no barrier after it (below)
                completed = true;
                break;
            }
            if (!grid_barrier(a.bar)) break;
        }
        if (__syncthreads_or(bad_type) && threadIdx.x == 0) atomicOr(&st->flags, kStBadIndex);
        if (threadIdx.x == 0 && ld_volatile(&a.bar->abort)) atomicOr(&st->flags, kStBarrierTimeout);
        // the last block to leave: after a completed launch it hands the pending rebuild
        // request to the next launch (or the per-step kernels) — every block has written its
        // part by then, so the last body needs no grid barrier of its own — and it mirrors
        // the final status into host memory, so the host reads it without a copy of its own
        if (threadIdx.x == 0) {
            // a launch that wrote host arrays orders them (its block's writes, by the barrier
            // above) before its arrival at the system scope: the host, once it sees the
            // launch's sequence number in the status mirror, reads them without waiting for
            // the launch to retire
            if (HOST_IO && cmd.hout[0]) __threadfence_system();
            else __threadfence();
            if (atomicAdd(&a.bar->exits, 1u) == gridDim.x - 1u) {
                a.bar->exits = 0u;  // (every block has counted itself: before the status goes out)
                __threadfence();
                if (completed) {  // the same in every block (all complete, or all left early)
                    st->rebuild = ld_volatile(&st->rb[cmd.bodies & 1]);
                    st->rb[0] = 0u;
                    st->rb[1] = 0u;
                }
                if (a.st_mirror) {
                    const volatile uint32_t* src = reinterpret_cast<const volatile uint32_t*>(st);
                    volatile uint32_t* dst = reinterpret_cast<volatile uint32_t*>(a.st_mirror);
                    constexpr int kSeqWord = (int)(offsetof(DevStatus, seq) / sizeof(uint32_t));
                    for (int k = 0; k < kSeqWord; ++k) dst[k] = src[k];
                    __threadfence_system();
                    dst[kSeqWord] = cmd.seq;  // after every other word
                    __threadfence_system();
                }
            }
        }
        if (!HOST_IO || a.req == nullptr) break;
        // host session: warp 0 of block 0 waits (at most idle_ns) for the host's next
        // request and copies it, one 8-byte word per lane (one round trip over the host
        // link), into the barrier's command; every block reads it after a grid barrier
        if (blockIdx.x == 0 && threadIdx.x < 32) {
            uint32_t go = 0u;
            if (threadIdx.x == 0 && !ld_volatile(&a.bar->abort)) {
                const unsigned long long t0 = global_ns();
                for (long long k = 1;; ++k) {
                    // (relaxed polls; an acquire at the system scope per poll measured
                    // several microseconds slower to see the host's store)
                    const uint32_t v = *(const volatile uint32_t*)&a.req->seq;
                    if (v != cmd.seq && v != 0u) {
                        go = v;
                        break;
                    }
                    if ((k & 63) == 0 && (global_ns() - t0 > a.idle_ns || k > kServeSpinLimit)) break;
                }
                // the host's stores before its store of the sequence number are visible
                // to the loads after this fence
                asm volatile("fence.acq_rel.sys;" ::: "memory");
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            __syncwarp();  // lane 0's fence before every lane's loads of the request
            constexpr int kReqWords = (int)(sizeof(HostRequest) / sizeof(unsigned long long));
            if (go && threadIdx.x < kReqWords)
                reinterpret_cast<unsigned long long*>(&a.bar->req)[threadIdx.x] =
                    *(reinterpret_cast<const volatile unsigned long long*>(a.req) + threadIdx.x);
            __syncwarp();
            if (threadIdx.x == 0) {
                if (go && a.bar->req.quit) go = 0u;
                if (go) {
                    const HostRequest& r = a.bar->req;
                    RunCmd& c = a.bar->cmd;
                    c.bodies = r.bodies;
                    c.closing = 1;
                    c.prologue = 3;
                    c.reuse_ok = r.reuse_ok;
                    c.rebuild0 = 0u;
                    c.seq = go;
                    c.step0 = r.step0;
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        c.hin[k] = r.hin[k];
                        c.hout[k] = r.hout[k];
                    }
                }
                *(volatile uint32_t*)&a.bar->go = go;
            }
        }
        if (!grid_barrier(a.bar)) break;
        // the command into shared memory, one 8-byte word per thread (L2, after the barrier)
        if (threadIdx.x == 0) serve_go = __ldcg(&a.bar->go);
        constexpr int kCmdWords = (int)(sizeof(RunCmd) / sizeof(unsigned long long));
        if (threadIdx.x < kCmdWords)
            reinterpret_cast<unsigned long long*>(&cmd)[threadIdx.x] =
                __ldcg(reinterpret_cast<const unsigned long long*>(&a.bar->cmd) + threadIdx.x);
        __syncthreads();
        if (!serve_go || cmd.bodies < 1) break;
    }
}
#endif

}  // namespace oxg
