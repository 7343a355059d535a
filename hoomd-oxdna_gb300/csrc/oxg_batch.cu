// oxg_batch.cu - batched independent replicas (many small systems, one launch).
//
// Each CTA owns a *tile*: one or more whole replicas whose particles it keeps in
// shared memory for the whole run (state, forces, frames, exclusions, bonds and the
// replicas' parameter blocks). A run of n steps is one persistent launch per chunk:
// inside it every step is prep/step-one -> forces -> step-two, separated only by
// __syncthreads, with no grid-wide synchronisation and no neighbour list (all pairs
// of each replica are tested; replicas are small). Heavy terms are compacted through
// shared-memory queues so they run with all lanes busy. Tiles are built on the host by
// first-fit-decreasing packing of the replicas by size; the tile capacity and the CTA
// size are chosen by an autotuner (oxg_batch_tune) that times short trial runs.
//
// Per replica: its own periodic box, parameters (its own context, e.g. temperature-
// dependent stacking and Debye-Hueckel) and bath temperature; the integrator is the
// single-system engine's (same functions), with the replica's seed and local particle
// indices as the Philox key/tag, so a replica reproduces a single-system run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/oxdna_gb300.h"
#include "oxg_internal.h"
#define OXG_DEVICE_FUNCTIONS_ONLY
#include "oxg_kernels.cuh"

using namespace oxg;

namespace {

#define BCUDA(call)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return internal_set_error(OXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kBatchMaxTile = 512;   // particles per tile (shared-memory bound)
constexpr int kBatchMaxReps = 32;    // replicas per tile

struct TileRep {
    int pstart, n, bstart, nb;   // global particle / bond ranges of the replica
    int loff, boff, tri_off, rep;  // tile-local particle / bond offsets, pair-index offset
    float3 L, invL;
    float kT;
    uint32_t seed_lo, seed_hi;
    float rlist2;  // (largest cutoff of the replica's terms + skin)^2
};

struct BatchArgs {
    int n_tiles;
    const int4* tiles;      // (first entry in rep_list, replicas, particles, bonds)
    const int* rep_list;
    const int4* rep_info;   // (particle start, n, bond start, n bonds)
    const float4* rep_box;  // (Lx, Ly, Lz, kT)
    const uint2* rep_seed;
    const unsigned char* params;
    int param_stride;
    int param_bytes;        // bytes to stage per replica
    float4 *pos, *pos_lo, *quat, *vel, *angmom;
    const float* charge;
    const int4* bonds;      // replica-local (A, B, type)
    const int4* excl;       // replica-local partners (-1 = none)
    uint32_t mask;
    int bonded;
    float dt, gamma, gamma_r;
    float3 inertia;
    unsigned long long step0;
    int nsteps;
    int resume;             // continue a run: accel / tnet hold the last step two's values
    float4* accel;          // (F + F_bath) / m after the last step two
    float4* tnet;           // T + T_bath after the last step two
    int max_reps, tile_cap, qcap;
    int plist_cap;          // tile pair-list capacity
    float skin;             // pair-list skin (rebuilt after a move of skin / 2)
    double* energy;         // [replica][9] (compute mode)
    float4* force_out;      // compute mode (may be null)
    float4* torque_out;
    uint32_t* status;
};

// shared-memory carve-up of one tile
struct Smem {
    TileRep* reps;
    unsigned char* params;
    float4 *x, *xl, *q, *v, *p, *f, *t;
    float4 *fa1, *fa2, *fa3;
    int4 *ex, *bd;
    int* rep_of;
    int* queue;  // kNQ * qcap entries: (i << 16) | j
    int* qcnt;
    int* nl;       // [0] pairs in plist, -1 = no list (all pairs tested every step)
    int* plist;    // tile pair list (pi << 16) | pj, pi < pj
    float4* xref;  // positions at the last list build
    double* eacc;  // [max_reps][9]
};

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t smem_bytes(int max_reps, int tile_cap, int qcap, int stride,
                                             bool energy, int plist_cap)
{
    size_t b = a16(sizeof(TileRep) * max_reps);
    b += a16((size_t)stride * max_reps);
    b += 10 * sizeof(float4) * (size_t)tile_cap;
    b += 2 * sizeof(int4) * (size_t)tile_cap;
    b += a16(sizeof(int) * tile_cap);
    b += a16(sizeof(int) * (size_t)kNQ * qcap);
    b += 32;  // queue counters (8 ints, kNQ used)
    b += 16;  // list counters
    b += a16(sizeof(int) * (size_t)plist_cap);
    b += sizeof(float4) * (size_t)tile_cap;
    if (energy) b += a16(sizeof(double) * 9 * max_reps);
    return b;
}

__device__ inline Smem carve(unsigned char* base, const BatchArgs& a, bool energy)
{
    Smem s;
    size_t o = 0;
    s.reps = reinterpret_cast<TileRep*>(base + o);
    o += a16(sizeof(TileRep) * a.max_reps);
    s.params = base + o;
    o += a16((size_t)a.param_bytes * a.max_reps);
    float4* f4 = reinterpret_cast<float4*>(base + o);
    const int P = a.tile_cap;
    s.x = f4;
    s.xl = f4 + P;
    s.q = f4 + 2 * P;
    s.v = f4 + 3 * P;
    s.p = f4 + 4 * P;
    s.f = f4 + 5 * P;
    s.t = f4 + 6 * P;
    s.fa1 = f4 + 7 * P;
    s.fa2 = f4 + 8 * P;
    s.fa3 = f4 + 9 * P;
    o += 10 * sizeof(float4) * (size_t)P;
    s.ex = reinterpret_cast<int4*>(base + o);
    s.bd = s.ex + P;
    o += 2 * sizeof(int4) * (size_t)P;
    s.rep_of = reinterpret_cast<int*>(base + o);
    o += a16(sizeof(int) * P);
    s.queue = reinterpret_cast<int*>(base + o);
    o += a16(sizeof(int) * (size_t)kNQ * a.qcap);
    s.qcnt = reinterpret_cast<int*>(base + o);
    o += 32;
    s.nl = reinterpret_cast<int*>(base + o);
    o += 16;
    s.plist = reinterpret_cast<int*>(base + o);
    o += a16(sizeof(int) * (size_t)a.plist_cap);
    s.xref = reinterpret_cast<float4*>(base + o);
    o += sizeof(float4) * (size_t)a.tile_cap;
    s.eacc = energy ? reinterpret_cast<double*>(base + o) : nullptr;
    return s;
}

__device__ inline Frame frame_of(const Smem& s, int p)
{
    Frame f;
    f.a1 = mk3(s.fa1[p].x, s.fa1[p].y, s.fa1[p].z);
    f.a2 = mk3(s.fa2[p].x, s.fa2[p].y, s.fa2[p].z);
    f.a3 = mk3(s.fa3[p].x, s.fa3[p].y, s.fa3[p].z);
    return f;
}

__device__ inline void sm_add(float4* arr, int p, float3 v, float w)
{
    atomicAdd(&arr[p].x, v.x);
    atomicAdd(&arr[p].y, v.y);
    atomicAdd(&arr[p].z, v.z);
    if (w != 0.f) atomicAdd(&arr[p].w, w);
}

template <bool ENERGY>
__device__ inline void scatter_pair(const Smem& s, int pi, int pj, int r, const PairAcc& acc,
                                    float e, int term)
{
    sm_add(s.f, pi, acc.fi, ENERGY ? 0.5f * e : 0.f);
    sm_add(s.f, pj, -acc.fi, ENERGY ? 0.5f * e : 0.f);
    sm_add(s.t, pi, acc.ti, 0.f);
    sm_add(s.t, pj, acc.tj, 0.f);
    if (ENERGY && e != 0.f) atomicAdd(&s.eacc[r * 9 + term], (double)e);
}

__device__ inline float3 rep_delta(const Smem& s, const TileRep& R, int pi, int pj)
{
    const float4 hi_i = s.x[pi], hi_j = s.x[pj], lo_i = s.xl[pi], lo_j = s.xl[pj];
    return image_delta(hi_i, lo_i, hi_j, lo_j, R.L, R.invL);
}

// the heavy term q of the tile pair (pi, pj) of replica r (block-cooperative caller)
template <bool ENERGY>
__device__ __noinline__ void batch_heavy(const Smem& s, const BatchArgs& a, int q, int pi, int pj, int r)
{
    const TileRep& R = s.reps[r];
    ParamView P;
    P.b = s.params + (size_t)r * a.param_bytes;
    const ParamHeader& H = P.h();
    const float3 dr = rep_delta(s, R, pi, pj);
    const float3 rc = -dr;
    const int pidx = __float_as_int(s.x[pi].w) * kMaxTypes + __float_as_int(s.x[pj].w);
    const Frame fi = frame_of(s, pi), fj = frame_of(s, pj);
    PairAcc acc;
    acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
    float e = 0.f;
    int term = kHBond;
    BBGeom g;
    if (q == kQHB) {
        const DHBond& ph = P.term<DHBond>(kHBond, pidx);
        if (bb_geometry(rc, fi, fj, ph.base, g)) {
            RadialF1 Rr{ph.f1, H.hb_eps[pidx], H.hb_shift[pidx]};
            e = bb_term<false>(g, fi, fj, ph.t1, ph.t23, ph.t4, ph.t78, true, Rr, acc);
        }
    } else if (q == kQCS) {
        term = kCross;
        const DCross& pc = P.term<DCross>(kCross, pidx);
        if (bb_geometry(rc, fi, fj, pc.base, g)) {
            RadialF2 Rr{pc.f2};
            e = bb_term<true>(g, fi, fj, pc.t1, pc.t23, pc.t4, pc.t78, pc.t4_enabled != 0, Rr, acc);
        }
    } else if (q == kQHBX || q == kQHBX0) {
        term = kHBCross;
        const DHBCross& px = P.term<DHBCross>(kHBCross, pidx);
        if (bb_geometry(rc, fi, fj, px.base, g)) {
            RadialF1 R1{px.f1, H.hbx_eps[pidx], H.hbx_shift[pidx]};
            e = bb_term<false>(g, fi, fj, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1, acc);
            RadialF2 R2{px.f2};
            e += bb_term<true>(g, fi, fj, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2, acc);
        }
    } else {
        term = kCoax;
        e = coax_term(P.term<DCoax>(kCoax, pidx), rc, fi, fj, acc);
    }
    scatter_pair<ENERGY>(s, pi, pj, r, acc, e, term);
}

// Phase-A work of one pair (pi < pj) of replica r: the cheap terms (excluded volume,
// Debye) inline, the zero-factor tests of the heavy ones; returns the heavy terms the
// pair needs (bit q: queue q), which the caller appends warp by warp.
template <bool ENERGY>
__device__ __forceinline__ uint32_t pair_a(const Smem& s, const BatchArgs& a, int r, int pi, int pj)
{
    const TileRep& R = s.reps[r];
    const int4 ex = s.ex[pi];
    if (ex.x == pj || ex.y == pj || ex.z == pj || ex.w == pj) return 0u;
    const float3 dr = rep_delta(s, R, pi, pj);
    const float rsq = dot(dr, dr);
    ParamView P;
    P.b = s.params + (size_t)r * a.param_bytes;
    const ParamHeader& H = P.h();
    if (!(rsq < H.rcutsq_max)) return 0u;
    const int pidx = __float_as_int(s.x[pi].w) * kMaxTypes + __float_as_int(s.x[pj].w);
    const Frame fi = frame_of(s, pi), fj = frame_of(s, pj);
    const float3 rc = -dr;
    const uint32_t mask = a.mask;
    PairAcc acc;
    acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
    float ev = 0.f, ed = 0.f;
    bool inl = false;
    if (mask & (1u << kExcVol)) {
        const DExcVol& pe = P.term<DExcVol>(kExcVol, pidx);
        if (rsq < pe.rcutsq) {
            ev = excvol_term(pe, rc, fi, fj, acc);
            inl = true;
        }
    }
    if (mask & (1u << kDebye)) {
        const DDebye& pd = P.term<DDebye>(kDebye, pidx);
        if (rsq < pd.rcutsq) {
            const float ci = a.charge[R.pstart + pi - R.loff], cj = a.charge[R.pstart + pj - R.loff];
            ed = debye_term(pd, rc, fi, fj, ci, cj, acc);
            inl = true;
        }
    }
    if (inl) {
        scatter_pair<ENERGY>(s, pi, pj, r, acc, ev + ed, kExcVol);
        if (ENERGY && ed != 0.f) {  // book the Debye part under its own term
            atomicAdd(&s.eacc[r * 9 + kExcVol], -(double)ed);
            atomicAdd(&s.eacc[r * 9 + kDebye], (double)ed);
        }
    }
    bool want[kNQ] = {};
    BBGeom g;
    bool gv = false;
    if (mask & (1u << kHBond)) {
        const DHBond& ph = P.term<DHBond>(kHBond, pidx);
        if (rsq < ph.rcutsq && H.hb_eps[pidx] != 0.f) {
            gv = bb_geometry(rc, fi, fj, ph.base, g);
            RadialF1 Rr{ph.f1, H.hb_eps[pidx], H.hb_shift[pidx]};
            want[kQHB] = gv && bb_support<false>(g, ph.t1, ph.t23, ph.t4, ph.t78, true, Rr);
        }
    }
    if (mask & (1u << kCross)) {
        const DCross& pc = P.term<DCross>(kCross, pidx);
        if (rsq < pc.rcutsq) {
            if (!gv || !H.hb_cs_same_site) gv = bb_geometry(rc, fi, fj, pc.base, g);
            RadialF2 Rr{pc.f2};
            want[kQCS] = gv && bb_support<true>(g, pc.t1, pc.t23, pc.t4, pc.t78, pc.t4_enabled != 0, Rr);
        }
    }
    if (mask & (1u << kHBCross)) {
        const DHBCross& px = P.term<DHBCross>(kHBCross, pidx);
        if (rsq < px.rcutsq && bb_geometry(rc, fi, fj, px.base, g)) {
            RadialF1 R1{px.f1, H.hbx_eps[pidx], H.hbx_shift[pidx]};
            RadialF2 R2{px.f2};
            want[kQHBX] = bb_support<false>(g, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1) ||
                          bb_support<true>(g, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2);
        }
    }
    if (mask & (1u << kCoax)) {
        const DCoax& pc = P.term<DCoax>(kCoax, pidx);
        want[kQCX] = rsq < pc.rcutsq && coax_support(pc, rc, fi, fj);
    }
    uint32_t bits = 0u;
#pragma unroll
    for (int q = 0; q < kNQ; ++q)
        if (want[q]) bits |= 1u << q;
    return bits;
}

// Append the warp's heavy-term pairs to the tile's queues: one shared atomic per warp and
// queue (all lanes call it; bits 0: nothing to append). A pair that does not fit is
// evaluated at once.
template <bool ENERGY>
__device__ __forceinline__ void queue_warp(const Smem& s, const BatchArgs& a, uint32_t bits, int r, int pi, int pj)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int q = 0; q < kNQ; ++q) {
        const bool w = (bits >> q) & 1u;
        const unsigned m = __ballot_sync(0xffffffffu, w);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&s.qcnt[q], __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (w) {
            const int slot = base + __popc(m & lt);
            if (slot < a.qcap) s.queue[q * a.qcap + slot] = (pi << 16) | pj;
            else batch_heavy<ENERGY>(s, a, q, pi, pj, r);  // queue full: evaluate here
        }
    }
}

// Pair k of the strictly upper triangles of the tile's replicas -> (replica, pi, pj).
__device__ __forceinline__ void tri_pair(const Smem& s, int nrep, int k, int& r, int& pi, int& pj)
{
    r = 0;
    while (r + 1 < nrep && k >= s.reps[r + 1].tri_off) ++r;
    const TileRep& R = s.reps[r];
    const int n = R.n;
    const int t = k - R.tri_off;
    // row i of the strictly upper triangle holding index t
    int i = (int)((2.f * n - 1.f - sqrtf((2.f * n - 1.f) * (2.f * n - 1.f) - 8.f * t)) * 0.5f);
    i = max(0, min(i, n - 2));
    while (i > 0 && t < i * (2 * n - i - 1) / 2) --i;
    while (i < n - 2 && t >= (i + 1) * (2 * n - i - 2) / 2) ++i;
    const int j = t - i * (2 * n - i - 1) / 2 + i + 1;
    pi = R.loff + i;
    pj = R.loff + j;
}

// Tile pair list: every bond-excluded-free pair within its replica's r_list; the list
// falls back to testing all pairs every step when it would exceed its capacity.
__device__ void build_list(const Smem& s, const BatchArgs& a, int nrep, int np, int total_pairs)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) s.nl[0] = 0;
    for (int p = tid; p < np; p += nt) s.xref[p] = s.x[p];
    __syncthreads();
    for (int k = tid; k < total_pairs; k += nt) {
        int r, pi, pj;
        tri_pair(s, nrep, k, r, pi, pj);
        const int4 ex = s.ex[pi];
        if (ex.x == pj || ex.y == pj || ex.z == pj || ex.w == pj) continue;
        const float3 dr = rep_delta(s, s.reps[r], pi, pj);
        if (!(dot(dr, dr) < s.reps[r].rlist2)) continue;
        const int slot = atomicAdd(&s.nl[0], 1);
        if (slot < a.plist_cap) s.plist[slot] = (pi << 16) | pj;
    }
    __syncthreads();
    if (tid == 0 && s.nl[0] > a.plist_cap) s.nl[0] = -1;
    __syncthreads();
}

// Forces of the whole tile into s.f / s.t (block-cooperative).
template <bool ENERGY>
__device__ void tile_forces(const Smem& s, const BatchArgs& a, int nrep, int np, int nb,
                            int total_pairs)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int p = tid; p < np; p += nt) {
        s.f[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        s.t[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        const Frame fr = quat_frame(s.q[p]);
        s.fa1[p] = make_float4(fr.a1.x, fr.a1.y, fr.a1.z, 0.f);
        s.fa2[p] = make_float4(fr.a2.x, fr.a2.y, fr.a2.z, 0.f);
        s.fa3[p] = make_float4(fr.a3.x, fr.a3.y, fr.a3.z, 0.f);
    }
    if (tid < kNQ) s.qcnt[tid] = 0;
    __syncthreads();
    // phase A: the tile's pair list (or every pair of every replica of the tile)
    const int npl = s.nl[0];
    // (loops run in whole warps: the queue appends are warp-wide)
    const int wbase0 = tid & ~31;
    if (npl >= 0) {
        for (int kb = wbase0; kb < npl; kb += nt) {
            const int k = kb + (tid & 31);
            uint32_t bits = 0u;
            int r = 0, pi = 0, pj = 0;
            if (k < npl) {
                const int v = s.plist[k];
                pi = v >> 16;
                pj = v & 0xffff;
                r = s.rep_of[pi];
                bits = pair_a<ENERGY>(s, a, r, pi, pj);
            }
            queue_warp<ENERGY>(s, a, bits, r, pi, pj);
        }
    } else {
        for (int kb = wbase0; kb < total_pairs; kb += nt) {
            const int k = kb + (tid & 31);
            uint32_t bits = 0u;
            int r = 0, pi = 0, pj = 0;
            if (k < total_pairs) {
                tri_pair(s, nrep, k, r, pi, pj);
                bits = pair_a<ENERGY>(s, a, r, pi, pj);
            }
            queue_warp<ENERGY>(s, a, bits, r, pi, pj);
        }
    }
    __syncthreads();
    // phase B: the queued heavy terms and the bonds as segments [HB | CS | HB+CS | coax |
    // bonds], each padded to whole warps, so that every warp evaluates 32 items of one
    // kind (term-uniform warps, no lane idle but in a segment's last warp)
    int cnt[kNQ + 1], seg[kNQ + 2];
    seg[0] = 0;
#pragma unroll
    for (int q = 0; q < kNQ; ++q) cnt[q] = min(s.qcnt[q], a.qcap);
    cnt[kNQ] = a.bonded ? nb : 0;
#pragma unroll
    for (int q = 0; q <= kNQ; ++q) seg[q + 1] = seg[q] + ((cnt[q] + 31) & ~31);
    const int lane = tid & 31;
    for (int wbase = (tid >> 5) * 32; wbase < seg[kNQ + 1]; wbase += nt) {
        int q = 0;
        while (q < kNQ && wbase >= seg[q + 1]) ++q;  // warp-uniform segment
        const int e = wbase - seg[q] + lane;
        if (e >= cnt[q]) continue;
        if (q < kNQ) {
            const int v = s.queue[q * a.qcap + e];
            const int pi = v >> 16, pj = v & 0xffff;
            batch_heavy<ENERGY>(s, a, q, pi, pj, s.rep_of[pi]);
            continue;
        }
        const int4 bd = s.bd[e];
        const int A = bd.x, B = bd.y, r = s.rep_of[A];
        const TileRep& R = s.reps[r];
        ParamView P;
        P.b = s.params + (size_t)r * a.param_bytes;
        const float3 Rcf = rep_delta(s, R, B, A);
        const float4 qA = s.q[A], qB = s.q[B];
        BondAcc acc;
        bonded_pair<false>(P.bonded(bd.z), make_double3(Rcf.x, Rcf.y, Rcf.z),
                    make_double4_32a(qA.x, qA.y, qA.z, qA.w), make_double4_32a(qB.x, qB.y, qB.z, qB.w),
                    __float_as_int(s.x[A].w), __float_as_int(s.x[B].w), acc);
        const float eh = ENERGY ? (float)(0.5 * (acc.e[0] + acc.e[1] + acc.e[2])) : 0.f;
        sm_add(s.f, A, -acc.fB, eh);
        sm_add(s.f, B, acc.fB, eh);
        sm_add(s.t, A, acc.tA, 0.f);
        sm_add(s.t, B, acc.tB, 0.f);
        if (ENERGY) {
            atomicAdd(&s.eacc[r * 9 + kNTerms + 0], acc.e[0]);
            atomicAdd(&s.eacc[r * 9 + kNTerms + 1], acc.e[1]);
            atomicAdd(&s.eacc[r * 9 + kNTerms + 2], acc.e[2]);
        }
    }
    __syncthreads();
}

template <bool ENERGY>
__global__ void __launch_bounds__(256) k_batch(BatchArgs a)
{
    extern __shared__ float4 smem_batch[];
    const Smem s = carve(reinterpret_cast<unsigned char*>(smem_batch), a, ENERGY);
    const int4 tile = a.tiles[blockIdx.x];
    const int nrep = tile.y, np = tile.z, nb = tile.w;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) {
        int loff = 0, boff = 0, tri = 0;
        for (int r = 0; r < nrep; ++r) {
            const int rep = a.rep_list[tile.x + r];
            const int4 info = a.rep_info[rep];
            const float4 box = a.rep_box[rep];
            const uint2 sd = a.rep_seed[rep];
            TileRep R;
            R.pstart = info.x;
            R.n = info.y;
            R.bstart = info.z;
            R.nb = info.w;
            R.loff = loff;
            R.boff = boff;
            R.tri_off = tri;
            R.rep = rep;
            R.L = mk3(box.x, box.y, box.z);
            R.invL = mk3(1.f / box.x, 1.f / box.y, 1.f / box.z);
            R.kT = box.w;
            R.seed_lo = sd.x;
            R.seed_hi = sd.y;
            R.rlist2 = 0.f;
            s.reps[r] = R;
            loff += info.y;
            boff += info.w;
            tri += info.y * (info.y - 1) / 2;
        }
        s.reps[nrep].tri_off = tri;  // sentinel (max_reps > nrep guaranteed by the host)
    }
    __syncthreads();
    const int total_pairs = s.reps[nrep].tri_off;
    // stage parameters and state
    const int words = a.param_bytes / 16;
    for (int r = 0; r < nrep; ++r) {
        const float4* src = reinterpret_cast<const float4*>(a.params + (size_t)s.reps[r].rep * a.param_stride);
        float4* dst = reinterpret_cast<float4*>(s.params + (size_t)r * a.param_bytes);
        for (int k = tid; k < words; k += nt) dst[k] = src[k];
        const TileRep R = s.reps[r];
        for (int i = tid; i < R.n; i += nt) {
            const int g = R.pstart + i, p = R.loff + i;
            s.x[p] = a.pos[g];
            s.xl[p] = a.pos_lo[g];
            s.q[p] = a.quat[g];
            s.v[p] = a.vel[g];
            s.p[p] = a.angmom[g];
            s.rep_of[p] = r;
            const int4 e = a.excl[g];
            s.ex[p] = make_int4(e.x >= 0 ? e.x + R.loff : -1, e.y >= 0 ? e.y + R.loff : -1,
                                e.z >= 0 ? e.z + R.loff : -1, e.w >= 0 ? e.w + R.loff : -1);
        }
        for (int b = tid; b < R.nb; b += nt) {
            const int4 bd = a.bonds[R.bstart + b];
            s.bd[R.boff + b] = make_int4(bd.x + R.loff, bd.y + R.loff, bd.z, 0);
        }
    }
    if (ENERGY)
        for (int k = tid; k < 9 * nrep; k += nt) s.eacc[k] = 0.0;
    __syncthreads();
    if (tid < nrep) {
        ParamView P;
        P.b = s.params + (size_t)tid * a.param_bytes;
        const float rl = sqrtf(P.h().rcutsq_max) + a.skin;
        s.reps[tid].rlist2 = rl * rl;
    }
    __syncthreads();
    build_list(s, a, nrep, np, total_pairs);
    const float half_skin2 = 0.25f * a.skin * a.skin;
    auto moved_far = [&](int p) {
        const TileRep& R = s.reps[s.rep_of[p]];
        const float4 x = s.x[p], x0 = s.xref[p];
        const float3 d = min_image(mk3(x.x - x0.x, x.y - x0.y, x.z - x0.z), R.L, R.invL);
        return dot(d, d) > half_skin2;
    };

    if (a.nsteps == 0 || !a.resume) tile_forces<ENERGY>(s, a, nrep, np, nb, total_pairs);
    if (a.nsteps == 0) {  // compute mode: forces and energies out
        for (int r = 0; r < nrep; ++r) {
            const TileRep R = s.reps[r];
            for (int i = tid; i < R.n; i += nt) {
                if (a.force_out) a.force_out[R.pstart + i] = s.f[R.loff + i];
                if (a.torque_out) a.torque_out[R.pstart + i] = s.t[R.loff + i];
            }
            if (ENERGY)
                for (int k = tid; k < 9; k += nt) a.energy[(size_t)R.rep * 9 + k] = s.eacc[r * 9 + k];
        }
        return;
    }
    bool bad = false;
    // first step one: accelerations of the last step two (resume) or, at the start of
    // a run, from the forces alone (prepRun: no bath)
    for (int p = tid; p < np; p += nt) {
        PState st{s.x[p], s.xl[p], s.v[p], s.q[p], s.p[p]};
        const TileRep& R = s.reps[s.rep_of[p]];
        float4 ac, tn;
        if (a.resume) {
            const int g = R.pstart + (p - R.loff);
            ac = a.accel[g];
            tn = a.tnet[g];
        } else {
            const float minv = 1.f / st.v.w;
            const float4 F = s.f[p], T = s.t[p];
            ac = make_float4(F.x * minv, F.y * minv, F.z * minv, 0.f);
            tn = make_float4(T.x, T.y, T.z, 0.f);
        }
        bad |= !step_one_pure(st, ac, tn, a.dt, R.L, a.inertia);
        s.x[p] = st.x;
        s.xl[p] = st.xl;
        s.v[p] = st.v;
        s.q[p] = st.q;
        s.p[p] = st.p;
    }
    bool far = false;
    for (int p = tid; p < np; p += nt) far |= moved_far(p);
    if (__syncthreads_or(far)) build_list(s, a, nrep, np, total_pairs);
    for (int step = 0; step < a.nsteps; ++step) {
        tile_forces<false>(s, a, nrep, np, nb, total_pairs);
        const unsigned long long ts = a.step0 + (unsigned long long)step + 1ull;
        const bool last = step == a.nsteps - 1;
        for (int p = tid; p < np; p += nt) {
            const int r = s.rep_of[p];
            const TileRep& R = s.reps[r];
            PState st{s.x[p], s.xl[p], s.v[p], s.q[p], s.p[p]};
            float4 ac, tn;
            step_two_pure(st, s.f[p], s.t[p], (uint32_t)(p - R.loff), ts, R.seed_lo, R.seed_hi, a.dt,
                          R.kT, a.gamma, a.gamma_r, a.inertia, ac, tn);
            if (!last) {
                bad |= !step_one_pure(st, ac, tn, a.dt, R.L, a.inertia);
            } else {
                const int g = R.pstart + (p - R.loff);
                a.accel[g] = ac;
                a.tnet[g] = tn;
            }
            s.x[p] = st.x;
            s.xl[p] = st.xl;
            s.v[p] = st.v;
            s.q[p] = st.q;
            s.p[p] = st.p;
        }
        __syncthreads();
        bool far_s = false;
        for (int p = tid; p < np; p += nt) far_s |= moved_far(p);
        if (__syncthreads_or(far_s) && !last) build_list(s, a, nrep, np, total_pairs);
    }
    // write the state back
    for (int r = 0; r < nrep; ++r) {
        const TileRep R = s.reps[r];
        for (int i = tid; i < R.n; i += nt) {
            const int g = R.pstart + i, p = R.loff + i;
            a.pos[g] = s.x[p];
            a.pos_lo[g] = s.xl[p];
            a.quat[g] = s.q[p];
            a.vel[g] = s.v[p];
            a.angmom[g] = s.p[p];
        }
    }
    if (__syncthreads_or(bad) && tid == 0) atomicOr(a.status, kStNonFinite);
}

template <class T>
int dalloc_b(T** p, size_t n)
{
    *p = nullptr;
    BCUDA(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
    return OXG_OK;
}
template <class T>
void dfree_b(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

struct oxg_batch {
    int R = 0, N = 0, NB = 0;
    // per replica, copied from its context at creation
    std::vector<std::vector<unsigned char>> blocks;
    std::vector<uint32_t> present;
    std::vector<int> ntypes;
    std::vector<char> bonded_ok;
    std::vector<int> pstart, n, bstart, nb;
    std::vector<float> box;  // 3 per replica
    std::vector<double> kT;
    cudaStream_t stream = nullptr;
    // device
    float4 *pos = nullptr, *pos_lo = nullptr, *quat = nullptr, *vel = nullptr, *angmom = nullptr;
    float4 *accel = nullptr, *tnet = nullptr;
    float* charge = nullptr;
    int4 *bonds = nullptr, *excl = nullptr;
    int4* rep_info = nullptr;
    float4* rep_box = nullptr;
    uint2* rep_seed = nullptr;
    unsigned char* params = nullptr;
    int param_stride = 0, param_bytes = 0;
    int4* tiles = nullptr;
    int* rep_list = nullptr;
    int n_tiles = 0, max_reps = 0, tile_cap = 0, threads = 128, qcap = 0;
    double* energy = nullptr;
    uint32_t* status = nullptr;
    // integrator
    double dt = 0.003, gamma = 1.0, gamma_r = 1.0;
    uint64_t seed = 1;
    uint32_t mask = 0;
    int bonded = 1;
    bool integ_set = false;
    unsigned long long timestep = 0;
    bool tuned = false;
    double tune_ms = 0.0;
};

namespace {

int upload_params(oxg_batch* b)
{
    const std::vector<std::vector<unsigned char>>& blocks = b->blocks;
    size_t mx = 0;
    for (int r = 0; r < b->R; ++r) mx = std::max(mx, blocks[r].size());
    const int stride = (int)((mx + 255) & ~size_t(255));
    std::vector<unsigned char> all((size_t)stride * b->R, 0);
    for (int r = 0; r < b->R; ++r) std::memcpy(all.data() + (size_t)stride * r, blocks[r].data(), blocks[r].size());
    dfree_b(b->params);
    int rc = dalloc_b(&b->params, all.size());
    if (rc) return rc;
    BCUDA(cudaMemcpy(b->params, all.data(), all.size(), cudaMemcpyHostToDevice));
    b->param_stride = stride;
    b->param_bytes = (int)((mx + 15) & ~size_t(15));
    return OXG_OK;
}

// First-fit-decreasing packing of replicas into tiles of at most `cap` particles.
int build_tiles(oxg_batch* b, int cap)
{
    std::vector<int> order(b->R);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->n[x] > b->n[y]; });
    std::vector<std::vector<int>> tiles;
    std::vector<int> load, bload;
    for (int r : order) {
        if (b->n[r] > cap)
            return internal_set_error(OXG_ERR_CAPACITY, "replica " + std::to_string(r) + " has " +
                                                            std::to_string(b->n[r]) + " particles, more than the tile capacity " +
                                                            std::to_string(cap));
        int t = -1;
        for (size_t k = 0; k < tiles.size(); ++k)
            if (load[k] + b->n[r] <= cap && bload[k] + b->nb[r] <= cap &&
                (int)tiles[k].size() < kBatchMaxReps - 1) {
                t = (int)k;
                break;
            }
        if (t < 0) {
            tiles.emplace_back();
            load.push_back(0);
            bload.push_back(0);
            t = (int)tiles.size() - 1;
        }
        tiles[t].push_back(r);
        load[t] += b->n[r];
        bload[t] += b->nb[r];
    }
    std::vector<int4> tinfo;
    std::vector<int> list;
    int mr = 0;
    for (size_t k = 0; k < tiles.size(); ++k) {
        tinfo.push_back(make_int4((int)list.size(), (int)tiles[k].size(), load[k], bload[k]));
        for (int r : tiles[k]) list.push_back(r);
        mr = std::max(mr, (int)tiles[k].size());
    }
    dfree_b(b->tiles);
    dfree_b(b->rep_list);
    int rc;
    if ((rc = dalloc_b(&b->tiles, tinfo.size())) || (rc = dalloc_b(&b->rep_list, list.size()))) return rc;
    BCUDA(cudaMemcpy(b->tiles, tinfo.data(), sizeof(int4) * tinfo.size(), cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->rep_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
    b->n_tiles = (int)tiles.size();
    b->max_reps = mr + 1;  // + sentinel entry
    b->tile_cap = cap;
    b->qcap = 3 * cap;
    return OXG_OK;
}

BatchArgs batch_args(oxg_batch* b, int nsteps, bool resume, float4* fout, float4* tout)
{
    BatchArgs a;
    a.n_tiles = b->n_tiles;
    a.tiles = b->tiles;
    a.rep_list = b->rep_list;
    a.rep_info = b->rep_info;
    a.rep_box = b->rep_box;
    a.rep_seed = b->rep_seed;
    a.params = b->params;
    a.param_stride = b->param_stride;
    a.param_bytes = b->param_bytes;
    a.pos = b->pos;
    a.pos_lo = b->pos_lo;
    a.quat = b->quat;
    a.vel = b->vel;
    a.angmom = b->angmom;
    a.charge = b->charge;
    a.bonds = b->bonds;
    a.excl = b->excl;
    a.mask = b->mask;
    a.bonded = b->bonded;
    a.dt = (float)b->dt;
    a.gamma = (float)b->gamma;
    a.gamma_r = (float)b->gamma_r;
    a.inertia = make_float3(1.f, 1.f, 1.f);
    a.step0 = b->timestep;
    a.nsteps = nsteps;
    a.resume = resume ? 1 : 0;
    a.accel = b->accel;
    a.tnet = b->tnet;
    a.max_reps = b->max_reps;
    a.tile_cap = b->tile_cap;
    a.qcap = b->qcap;
    a.plist_cap = 32 * b->tile_cap;
    a.skin = 0.4f;
    a.energy = b->energy;
    a.force_out = fout;
    a.torque_out = tout;
    a.status = b->status;
    return a;
}

int launch_batch(oxg_batch* b, int nsteps, bool resume, bool energy, float4* fout, float4* tout)
{
    const BatchArgs a = batch_args(b, nsteps, resume, fout, tout);
    const size_t sm = smem_bytes(b->max_reps, b->tile_cap, b->qcap, b->param_bytes, energy, 32 * b->tile_cap);
    if (sm > 227 * 1024)
        return internal_set_error(OXG_ERR_CAPACITY, "tile needs " + std::to_string(sm) + " bytes of shared memory");
    if (energy) {
        BCUDA(cudaFuncSetAttribute(k_batch<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_batch<true><<<b->n_tiles, b->threads, sm, b->stream>>>(a);
    } else {
        BCUDA(cudaFuncSetAttribute(k_batch<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_batch<false><<<b->n_tiles, b->threads, sm, b->stream>>>(a);
    }
    BCUDA(cudaGetLastError());
    return OXG_OK;
}

int ensure_ready(oxg_batch* b)
{
    if (!b->params) {
        int rc = upload_params(b);
        if (rc) return rc;
    }
    if (!b->tiles) {
        int rc = build_tiles(b, 256);
        if (rc) return rc;
    }
    return OXG_OK;
}

}  // namespace

extern "C" {

int oxg_batch_create(oxg_batch** out, int R, oxg_context* const* ctxs, const int32_t* n_particles,
                     const float* boxes, const int32_t* n_bonds, const int32_t* bonds)
{
    if (!out || R <= 0 || !ctxs || !n_particles || !boxes || !n_bonds)
        return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    *out = nullptr;
    oxg_batch* b = new oxg_batch();
    b->R = R;
    int N = 0, NB = 0;
    std::vector<int4> bnd, excl;
    for (int r = 0; r < R; ++r) {
        if (!ctxs[r] || n_particles[r] < 1 || n_bonds[r] < 0 || !(boxes[3 * r] > 0.f) ||
            !(boxes[3 * r + 1] > 0.f) || !(boxes[3 * r + 2] > 0.f)) {
            delete b;
            return internal_set_error(OXG_ERR_INVALID_ARG, "bad replica " + std::to_string(r));
        }
        b->pstart.push_back(N);
        b->n.push_back(n_particles[r]);
        b->bstart.push_back(NB);
        b->nb.push_back(n_bonds[r]);
        std::vector<int4> ex(n_particles[r], make_int4(-1, -1, -1, -1));
        for (int k = 0; k < n_bonds[r]; ++k) {
            const int32_t* bb = bonds + 3 * (size_t)(NB + k);
            const int A = bb[0], B = bb[1], t = bb[2];
            if (A < 0 || B < 0 || A >= n_particles[r] || B >= n_particles[r] || A == B || t < 0) {
                delete b;
                return internal_set_error(OXG_ERR_BAD_INDEX, "replica " + std::to_string(r) + " bond " +
                                                                 std::to_string(k) + " has an invalid index");
            }
            bnd.push_back(make_int4(A, B, t, 0));
            for (int pass = 0; pass < 2; ++pass) {
                int4& e = ex[pass ? B : A];
                const int o = pass ? A : B;
                if (e.x < 0) e.x = o;
                else if (e.y < 0) e.y = o;
                else if (e.z < 0) e.z = o;
                else if (e.w < 0) e.w = o;
                else {
                    delete b;
                    return internal_set_error(OXG_ERR_CAPACITY, "a particle has more than 4 bonds");
                }
            }
        }
        excl.insert(excl.end(), ex.begin(), ex.end());
        N += n_particles[r];
        NB += n_bonds[r];
        for (int d = 0; d < 3; ++d) b->box.push_back(boxes[3 * r + d]);
    }
    b->N = N;
    b->NB = NB;
    b->blocks.resize(R);
    for (int r = 0; r < R; ++r) {
        const int rc = internal_assemble_block(ctxs[r], b->blocks[r]);
        if (rc) {
            delete b;
            return rc;
        }
        if ((int)b->blocks[r].size() > kParamBlockMax) {
            delete b;
            return internal_set_error(OXG_ERR_CAPACITY, "parameter block too large");
        }
        b->present.push_back(internal_present_mask(ctxs[r]));
        b->ntypes.push_back(internal_n_types(ctxs[r]));
        b->bonded_ok.push_back(internal_bonded_complete(ctxs[r]) ? 1 : 0);
        ParamHeader H;
        std::memcpy(&H, b->blocks[r].data(), sizeof(H));
        for (int k = 0; k < n_bonds[r]; ++k)
            if (bnd[b->bstart[r] + k].z >= H.n_bond_types) {
                delete b;
                return internal_set_error(OXG_ERR_BAD_INDEX, "replica " + std::to_string(r) +
                                                                 " has a bond type outside its context");
            }
    }
    b->kT.assign(R, 0.1);
    int rc;
    if ((rc = dalloc_b(&b->pos, N)) || (rc = dalloc_b(&b->pos_lo, N)) || (rc = dalloc_b(&b->quat, N)) ||
        (rc = dalloc_b(&b->vel, N)) || (rc = dalloc_b(&b->angmom, N)) || (rc = dalloc_b(&b->charge, N)) ||
        (rc = dalloc_b(&b->accel, N)) || (rc = dalloc_b(&b->tnet, N)) ||
        (rc = dalloc_b(&b->bonds, std::max(1, NB))) || (rc = dalloc_b(&b->excl, N)) ||
        (rc = dalloc_b(&b->rep_info, R)) || (rc = dalloc_b(&b->rep_box, R)) ||
        (rc = dalloc_b(&b->rep_seed, R)) || (rc = dalloc_b(&b->energy, 9 * (size_t)R)) ||
        (rc = dalloc_b(&b->status, 1))) {
        oxg_batch_destroy(b);
        return rc;
    }
    std::vector<int4> info(R);
    for (int r = 0; r < R; ++r) info[r] = make_int4(b->pstart[r], b->n[r], b->bstart[r], b->nb[r]);
    cudaMemcpy(b->rep_info, info.data(), sizeof(int4) * R, cudaMemcpyHostToDevice);
    if (NB) cudaMemcpy(b->bonds, bnd.data(), sizeof(int4) * NB, cudaMemcpyHostToDevice);
    cudaMemcpy(b->excl, excl.data(), sizeof(int4) * N, cudaMemcpyHostToDevice);
    cudaMemset(b->status, 0, sizeof(uint32_t));
    std::vector<float4> z(N, make_float4(0.f, 0.f, 0.f, 0.f)), v(N, make_float4(0.f, 0.f, 0.f, 1.f)),
        q(N, make_float4(1.f, 0.f, 0.f, 0.f));
    std::vector<float> ch(N, 1.f);
    cudaMemcpy(b->pos, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b->pos_lo, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b->angmom, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b->vel, v.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b->quat, q.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(b->charge, ch.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    std::vector<float4> box(R);
    std::vector<uint2> sd(R, make_uint2(0u, 0u));
    for (int r = 0; r < R; ++r) box[r] = make_float4(b->box[3 * r], b->box[3 * r + 1], b->box[3 * r + 2], 0.f);
    cudaMemcpy(b->rep_box, box.data(), sizeof(float4) * R, cudaMemcpyHostToDevice);
    cudaMemcpy(b->rep_seed, sd.data(), sizeof(uint2) * R, cudaMemcpyHostToDevice);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        oxg_batch_destroy(b);
        return internal_set_error(OXG_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = b;
    return OXG_OK;
}

int oxg_batch_destroy(oxg_batch* b)
{
    if (!b) return OXG_OK;
    dfree_b(b->pos); dfree_b(b->pos_lo); dfree_b(b->quat); dfree_b(b->vel); dfree_b(b->angmom);
    dfree_b(b->accel); dfree_b(b->tnet);
    dfree_b(b->charge); dfree_b(b->bonds); dfree_b(b->excl); dfree_b(b->rep_info);
    dfree_b(b->rep_box); dfree_b(b->rep_seed); dfree_b(b->params); dfree_b(b->tiles);
    dfree_b(b->rep_list); dfree_b(b->energy); dfree_b(b->status);
    delete b;
    return OXG_OK;
}

int oxg_batch_set_stream(oxg_batch* b, void* stream)
{
    if (!b) return internal_set_error(OXG_ERR_INVALID_ARG, "null batch");
    b->stream = (cudaStream_t)stream;
    return OXG_OK;
}

int oxg_batch_set_state(oxg_batch* b, const float* pos_type, const float* pos_lo, const float* quat,
                        const float* vel, const float* angmom, const float* charge)
{
    if (!b) return internal_set_error(OXG_ERR_INVALID_ARG, "null batch");
    const size_t b4 = sizeof(float4) * b->N;
    if (pos_type) {
        for (int r = 0; r < b->R; ++r) {
            const int nt = b->ntypes[r];
            for (int i = 0; i < b->n[r]; ++i) {
                int t;
                std::memcpy(&t, pos_type + 4 * (size_t)(b->pstart[r] + i) + 3, sizeof(int));
                if (t < 0 || t >= nt)
                    return internal_set_error(OXG_ERR_BAD_INDEX, "replica " + std::to_string(r) +
                                                                     " has a particle type outside its context");
            }
        }
        BCUDA(cudaMemcpyAsync(b->pos, pos_type, b4, cudaMemcpyHostToDevice, b->stream));
        if (!pos_lo) BCUDA(cudaMemsetAsync(b->pos_lo, 0, b4, b->stream));
    }
    if (pos_lo) BCUDA(cudaMemcpyAsync(b->pos_lo, pos_lo, b4, cudaMemcpyHostToDevice, b->stream));
    if (quat) BCUDA(cudaMemcpyAsync(b->quat, quat, b4, cudaMemcpyHostToDevice, b->stream));
    if (vel) BCUDA(cudaMemcpyAsync(b->vel, vel, b4, cudaMemcpyHostToDevice, b->stream));
    if (angmom) BCUDA(cudaMemcpyAsync(b->angmom, angmom, b4, cudaMemcpyHostToDevice, b->stream));
    if (charge) BCUDA(cudaMemcpyAsync(b->charge, charge, sizeof(float) * b->N, cudaMemcpyHostToDevice, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return OXG_OK;
}

int oxg_batch_get_state(oxg_batch* b, float* pos_type, float* pos_lo, float* quat, float* vel,
                        float* angmom)
{
    if (!b) return internal_set_error(OXG_ERR_INVALID_ARG, "null batch");
    const size_t b4 = sizeof(float4) * b->N;
    if (pos_type) BCUDA(cudaMemcpyAsync(pos_type, b->pos, b4, cudaMemcpyDeviceToHost, b->stream));
    if (pos_lo) BCUDA(cudaMemcpyAsync(pos_lo, b->pos_lo, b4, cudaMemcpyDeviceToHost, b->stream));
    if (quat) BCUDA(cudaMemcpyAsync(quat, b->quat, b4, cudaMemcpyDeviceToHost, b->stream));
    if (vel) BCUDA(cudaMemcpyAsync(vel, b->vel, b4, cudaMemcpyDeviceToHost, b->stream));
    if (angmom) BCUDA(cudaMemcpyAsync(angmom, b->angmom, b4, cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    return OXG_OK;
}

int oxg_batch_set_integrator(oxg_batch* b, double dt, const double* kT, double gamma, double gamma_r,
                             uint64_t seed, uint32_t mask, int bonded)
{
    if (!b || !kT || !(dt > 0.0) || !(gamma >= 0.0) || !(gamma_r >= 0.0))
        return internal_set_error(OXG_ERR_INVALID_ARG, "bad integrator parameters");
    for (int r = 0; r < b->R; ++r) {
        if (mask & ~b->present[r])
            return internal_set_error(OXG_ERR_NO_PARAMS, "replica " + std::to_string(r) + " lacks a requested term");
        if (bonded && !b->bonded_ok[r])
            return internal_set_error(OXG_ERR_NO_PARAMS, "replica " + std::to_string(r) + " lacks bonded parameters");
        if (!(kT[r] >= 0.0)) return internal_set_error(OXG_ERR_INVALID_ARG, "negative kT");
    }
    b->dt = dt;
    b->gamma = gamma;
    b->gamma_r = gamma_r;
    b->seed = seed;
    b->mask = mask;
    b->bonded = bonded;
    b->kT.assign(kT, kT + b->R);
    std::vector<float4> box(b->R);
    std::vector<uint2> sd(b->R);
    for (int r = 0; r < b->R; ++r) {
        box[r] = make_float4(b->box[3 * r], b->box[3 * r + 1], b->box[3 * r + 2], (float)kT[r]);
        const uint64_t s = seed + (uint64_t)r;  // replica r runs with seed + r
        sd[r] = make_uint2((uint32_t)s, (uint32_t)(s >> 32));
    }
    BCUDA(cudaMemcpy(b->rep_box, box.data(), sizeof(float4) * b->R, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->rep_seed, sd.data(), sizeof(uint2) * b->R, cudaMemcpyHostToDevice));
    b->integ_set = true;
    return OXG_OK;
}

int oxg_batch_set_tiling(oxg_batch* b, int tile_particles, int threads)
{
    if (!b || tile_particles < 1 || tile_particles > kBatchMaxTile || (threads != 64 && threads != 128 && threads != 256))
        return internal_set_error(OXG_ERR_INVALID_ARG, "tile size must be 1..512, threads 64/128/256");
    b->threads = threads;
    return build_tiles(b, tile_particles);
}

int oxg_batch_run(oxg_batch* b, long nsteps)
{
    if (!b || nsteps < 0) return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    if (!b->integ_set) return internal_set_error(OXG_ERR_INVALID_ARG, "integrator not set");
    int rc = ensure_ready(b);
    if (rc) return rc;
    BCUDA(cudaMemsetAsync(b->status, 0, sizeof(uint32_t), b->stream));
    // chunks keep a single launch within a few hundred milliseconds
    const long chunk = 5000;
    for (long done = 0; done < nsteps;) {
        const int todo = (int)std::min(chunk, nsteps - done);
        if ((rc = launch_batch(b, todo, done > 0, false, nullptr, nullptr))) return rc;
        b->timestep += (unsigned long long)todo;
        done += todo;
    }
    uint32_t st = 0;
    BCUDA(cudaMemcpyAsync(&st, b->status, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
    BCUDA(cudaStreamSynchronize(b->stream));
    if (st & kStNonFinite) return internal_set_error(OXG_ERR_NONFINITE, "a replica reached a non-finite state");
    return OXG_OK;
}

int oxg_batch_compute(oxg_batch* b, uint32_t mask, int bonded, float* force, float* torque,
                      double* energies)
{
    if (!b) return internal_set_error(OXG_ERR_INVALID_ARG, "null batch");
    const uint32_t m0 = b->mask;
    const int b0 = b->bonded;
    for (int r = 0; r < b->R; ++r)
        if (mask & ~b->present[r])
            return internal_set_error(OXG_ERR_NO_PARAMS, "a replica lacks a requested term");
    if (bonded)
        for (int r = 0; r < b->R; ++r)
            if (!b->bonded_ok[r]) return internal_set_error(OXG_ERR_NO_PARAMS, "a replica lacks bonded parameters");
    b->mask = mask;
    b->bonded = bonded;
    int rc = ensure_ready(b);
    float4 *fd = nullptr, *td = nullptr;
    if (!rc) rc = dalloc_b(&fd, b->N);
    if (!rc) rc = dalloc_b(&td, b->N);
    if (!rc) rc = launch_batch(b, 0, false, true, fd, td);
    if (!rc) {
        const size_t b4 = sizeof(float4) * b->N;
        if (force) cudaMemcpyAsync(force, fd, b4, cudaMemcpyDeviceToHost, b->stream);
        if (torque) cudaMemcpyAsync(torque, td, b4, cudaMemcpyDeviceToHost, b->stream);
        if (energies) cudaMemcpyAsync(energies, b->energy, sizeof(double) * 9 * b->R, cudaMemcpyDeviceToHost, b->stream);
        if (cudaStreamSynchronize(b->stream) != cudaSuccess) rc = internal_set_error(OXG_ERR_CUDA, "batch compute");
    }
    dfree_b(fd);
    dfree_b(td);
    b->mask = m0;
    b->bonded = b0;
    return rc;
}

int oxg_batch_tune(oxg_batch* b, int trial_steps, int* tile_out, int* threads_out, double* ms_out)
{
    if (!b || trial_steps < 1) return internal_set_error(OXG_ERR_INVALID_ARG, "bad arguments");
    if (!b->integ_set) return internal_set_error(OXG_ERR_INVALID_ARG, "integrator not set");
    int rc = ensure_ready(b);
    if (rc) return rc;
    // keep the state: tuning runs advance it
    const size_t b4 = sizeof(float4) * b->N;
    float4* save[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float4* cur[5] = {b->pos, b->pos_lo, b->quat, b->vel, b->angmom};
    for (int k = 0; k < 5; ++k) {
        if ((rc = dalloc_b(&save[k], b->N))) return rc;
        BCUDA(cudaMemcpyAsync(save[k], cur[k], b4, cudaMemcpyDeviceToDevice, b->stream));
    }
    const unsigned long long ts0 = b->timestep;
    int max_n = *std::max_element(b->n.begin(), b->n.end());
    int best_tile = 0, best_threads = 0;
    double best = 1e300;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // fixed capacities, plus the ones that pack the particles into whole waves of one
    // tile per SM (1, 2 or 3 waves; 4% slack for the packing), rounded up to 16
    std::vector<int> caps = {64, 128, 192, 256, 384, 512};
    const int sms = internal_num_sms();
    for (int w = 1; w <= 3; ++w) {
        const double per = 1.04 * (double)b->N / (double)(w * sms);
        const int cap = ((int)std::ceil(per / 16.0)) * 16;
        if (cap >= max_n && cap <= kBatchMaxTile) caps.push_back(cap);
    }
    std::sort(caps.begin(), caps.end());
    caps.erase(std::unique(caps.begin(), caps.end()), caps.end());
    for (int cap : caps) {
        if (cap < max_n) continue;
        for (int th : {64, 128, 256}) {
            if (th > 2 * cap) continue;
            b->threads = th;
            if ((rc = build_tiles(b, cap))) break;
            const size_t sm = smem_bytes(b->max_reps, b->tile_cap, b->qcap, b->param_bytes, false, 32 * b->tile_cap);
            if (sm > 227 * 1024) continue;
            launch_batch(b, 2, false, false, nullptr, nullptr);  // warm-up
            cudaEventRecord(e0, b->stream);
            rc = launch_batch(b, trial_steps, false, false, nullptr, nullptr);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rc == OXG_OK && ms < best) {
                best = ms;
                best_tile = cap;
                best_threads = th;
            }
            for (int k = 0; k < 5; ++k)
                cudaMemcpyAsync(cur[k], save[k], b4, cudaMemcpyDeviceToDevice, b->stream);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int k = 0; k < 5; ++k) dfree_b(save[k]);
    b->timestep = ts0;
    if (best_tile == 0) return internal_set_error(OXG_ERR_CAPACITY, "no tile shape fits the largest replica");
    b->threads = best_threads;
    if ((rc = build_tiles(b, best_tile))) return rc;
    b->tuned = true;
    b->tune_ms = best;
    if (tile_out) *tile_out = best_tile;
    if (threads_out) *threads_out = best_threads;
    if (ms_out) *ms_out = best;
    BCUDA(cudaStreamSynchronize(b->stream));
    return OXG_OK;
}

}  // extern "C"
