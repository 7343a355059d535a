// oxg_engine.cu - host side of the GB300 oxDNA force engine and its C ABI
// (include/oxdna_gb300.h).
//
// oxg_context  holds the per-term, per-type-pair parameters (the reference's
//              param_type PODs, src/EvaluatorPairOxDNA*.h, src/OxDNABondedParams.h)
//              and their FP32 device block.
// oxg_system   is the resident-state engine that stands in for the HOOMD runtime:
//              SoA float4 state in HBM, a cell neighbour list with bond exclusions
//              and a buffer (HOOMD Cell nlist semantics, oxdna/model/dna1.py:307-309),
//              one fused force kernel per step and the Langevin / NO_SQUISH
//              integrator, replayed from a captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/oxdna_gb300.h"
#include "oxg_convert.h"
#include "oxg_internal.h"
#include "oxg_kernels.cuh"

using namespace oxg;

namespace {

thread_local std::string g_last_error;

int set_err(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

#define OXG_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return set_err(OXG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    OXG_CUDA(cudaMalloc((void**)p, n * sizeof(T)));
    return OXG_OK;
}
template <class T>
void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

int num_sms()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

// ======================================================================== context
template <class POD>
struct TermTable {
    bool any = false;
    POD p[kMaxPairs];
    double rcut[kMaxPairs];
    bool set[kMaxPairs];
    TermTable()
    {
        std::memset(p, 0, sizeof(p));
        for (int k = 0; k < kMaxPairs; ++k) {
            rcut[k] = 0.0;
            set[k] = false;
        }
    }
};

struct oxg_context {
    int device = 0;
    int n_types = 0;
    int n_bond_types = 0;
    TermTable<oxg_excvol_params> excvol;
    TermTable<oxg_hbond_params> hbond;
    TermTable<oxg_cross_params> cross;
    TermTable<oxg_hbondcross_params> hbx;
    TermTable<oxg_coax_params> coax;
    TermTable<oxg_debye_params> debye;
    std::vector<oxg_bonded_params> bonded;
    std::vector<bool> bonded_set;
    std::vector<unsigned char> block;  // host image of the device block
    unsigned char* d_block = nullptr;
    int block_bytes = 0;
    bool dirty = true;
    uint64_t version = 0;
    uint32_t* d_status = nullptr;
    cudaStream_t last_stream = nullptr;
    int first_error = OXG_OK;
    float4* conv = nullptr;  // oxg_pair_forces: FP32 copies of HOOMD's arrays (3 x conv_cap)
    int conv_cap = 0;
};

namespace {

template <class POD, class D>
bool add_term(const oxg_context* c, const TermTable<POD>& tt, int tid, ParamHeader& H,
              std::vector<unsigned char>& blk, float& rmax2, float& rshort2, bool is_short)
{
    if (!tt.any) return true;
    const int nt = c->n_types;
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nt; ++b)
            if (!tt.set[a * kMaxTypes + b]) return false;
    std::vector<D> d(kMaxPairs);
    std::memset(d.data(), 0, sizeof(D) * kMaxPairs);
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nt; ++b) {
            const int k = a * kMaxTypes + b;
            d[k] = to_dev(tt.p[k], tt.rcut[k]);
            rmax2 = std::max(rmax2, sq(tt.rcut[k]));
            if (is_short) rshort2 = std::max(rshort2, sq(tt.rcut[k]));
        }
    bool uniform = true;
    for (int a = 0; a < nt && uniform; ++a)
        for (int b = 0; b < nt; ++b)
            if (std::memcmp(&d[a * kMaxTypes + b], &d[0], sizeof(D)) != 0) {
                uniform = false;
                break;
            }
    const size_t off = align16(blk.size());
    const int count = uniform ? 1 : kMaxPairs;
    blk.resize(off + align16(sizeof(D) * count), 0);
    std::memcpy(blk.data() + off, d.data(), sizeof(D) * count);
    H.off[tid] = (int)off;
    H.stride[tid] = uniform ? 0 : (int)sizeof(D);
    H.present |= 1u << tid;
    return true;
}

// Host image of a context's FP32 parameter block (header, term structs, bonded).
int assemble_block(const oxg_context* c, std::vector<unsigned char>& blk)
{
    ParamHeader H;
    std::memset(&H, 0, sizeof(H));
    H.n_types = c->n_types;
    H.n_bond_types = c->n_bond_types;
    blk.assign(align16(sizeof(ParamHeader)), 0);
    float rmax2 = 0.f, rshort2 = 0.f;
    bool ok = add_term<oxg_excvol_params, DExcVol>(c, c->excvol, kExcVol, H, blk, rmax2, rshort2, true) &&
              add_term<oxg_hbond_params, DHBond>(c, c->hbond, kHBond, H, blk, rmax2, rshort2, true) &&
              add_term<oxg_cross_params, DCross>(c, c->cross, kCross, H, blk, rmax2, rshort2, true) &&
              add_term<oxg_hbondcross_params, DHBCross>(c, c->hbx, kHBCross, H, blk, rmax2, rshort2, true) &&
              add_term<oxg_coax_params, DCoax>(c, c->coax, kCoax, H, blk, rmax2, rshort2, true) &&
              add_term<oxg_debye_params, DDebye>(c, c->debye, kDebye, H, blk, rmax2, rshort2, false);
    if (!ok) return set_err(OXG_ERR_NO_PARAMS, "a term has parameters for some but not all type pairs");
    for (int k = 0; k < kMaxPairs; ++k) {
        if (c->hbond.any) {
            H.hb_eps[k] = (float)c->hbond.p[k].eps;
            H.hb_shift[k] = (float)(c->hbond.p[k].eps * c->hbond.p[k].shift_factor);
        }
        if (c->hbx.any) {
            H.hbx_eps[k] = (float)c->hbx.p[k].eps;
            H.hbx_shift[k] = (float)(c->hbx.p[k].eps * c->hbx.p[k].shift_factor);
        }
    }
    H.hb_cs_same_site = 0;
    if (c->hbond.any && c->cross.any) {
        bool same = true;
        for (int k = 0; k < kMaxPairs; ++k)
            for (int d = 0; d < 3; ++d)
                if (c->hbond.p[k].base_site[d] != c->cross.p[k].base_site[d]) same = false;
        H.hb_cs_same_site = same ? 1 : 0;
    }
    H.rcutsq_max = rmax2;
    H.rcutsq_short = rshort2;
    const size_t offb = align16(blk.size());
    std::vector<DBonded> bd(std::max(1, c->n_bond_types));
    for (int t = 0; t < c->n_bond_types; ++t)
        if (c->bonded_set[t]) bd[t] = to_dev(c->bonded[t]);
        else std::memset(&bd[t], 0, sizeof(DBonded));
    blk.resize(offb + align16(sizeof(DBonded) * bd.size()), 0);
    std::memcpy(blk.data() + offb, bd.data(), sizeof(DBonded) * bd.size());
    H.off_bonded = (int)offb;
    H.total_bytes = (int)blk.size();
    std::memcpy(blk.data(), &H, sizeof(H));
    if (blk.size() > (size_t)kParamBlockMax)
        return set_err(OXG_ERR_CAPACITY, "parameter block larger than the shared-memory budget");
    return OXG_OK;
}

int build_block(oxg_context* c)
{
    if (!c->dirty) return OXG_OK;
    std::vector<unsigned char> blk;
    const int arc = assemble_block(c, blk);
    if (arc) return arc;
    if ((int)blk.size() > c->block_bytes) {
        dfree(c->d_block);
        int rc = dalloc(&c->d_block, kParamBlockMax);
        if (rc) return rc;
    }
    OXG_CUDA(cudaMemcpy(c->d_block, blk.data(), blk.size(), cudaMemcpyHostToDevice));
    c->block = blk;
    c->block_bytes = (int)blk.size();
    c->dirty = false;
    c->version++;
    return OXG_OK;
}



template <class POD>
int set_pair(oxg_context* c, TermTable<POD>& tt, int ti, int tj, const POD* p, double rcut)
{
    if (!c || !p) return set_err(OXG_ERR_INVALID_ARG, "null context or parameters");
    if (ti < 0 || tj < 0 || ti >= c->n_types || tj >= c->n_types)
        return set_err(OXG_ERR_INVALID_ARG, "type index out of range");
    if (!(rcut >= 0.0)) return set_err(OXG_ERR_INVALID_ARG, "negative r_cut");
    for (int k : {ti * kMaxTypes + tj, tj * kMaxTypes + ti}) {
        tt.p[k] = *p;
        tt.rcut[k] = rcut;
        tt.set[k] = true;
    }
    tt.any = true;
    c->dirty = true;
    return OXG_OK;
}

}  // namespace

extern "C" {

const char* oxg_version(void) { return "oxdna_gb300 1.0 (sm_103a)"; }
const char* oxg_last_error(void) { return g_last_error.c_str(); }

const char* oxg_status_string(int s)
{
    switch (s) {
    case OXG_OK: return "ok";
    case OXG_ERR_INVALID_ARG: return "invalid argument";
    case OXG_ERR_CUDA: return "CUDA error";
    case OXG_ERR_NLIST_OVERFLOW: return "neighbour list overflow";
    case OXG_ERR_BAD_INDEX: return "index out of range";
    case OXG_ERR_TIMEOUT: return "device wait timed out";
    case OXG_ERR_NO_PARAMS: return "missing parameters";
    case OXG_ERR_CAPACITY: return "capacity exceeded";
    case OXG_ERR_NONFINITE: return "non-finite state";
    }
    return "unknown status";
}

int oxg_create(oxg_context** out, int n_types, int n_bond_types)
{
    if (!out) return set_err(OXG_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    if (n_types < 1 || n_types > kMaxTypes || n_bond_types < 0 || n_bond_types > kMaxBondTypes)
        return set_err(OXG_ERR_INVALID_ARG, "n_types must be 1..4 and n_bond_types 0..4");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return set_err(OXG_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    oxg_context* c = new oxg_context();
    cudaGetDevice(&c->device);
    c->n_types = n_types;
    c->n_bond_types = n_bond_types;
    c->bonded.assign(std::max(1, n_bond_types), oxg_bonded_params());
    std::memset(c->bonded.data(), 0, sizeof(oxg_bonded_params) * c->bonded.size());
    c->bonded_set.assign(std::max(1, n_bond_types), false);
    int rc = dalloc(&c->d_status, 1);
    if (rc) {
        delete c;
        return rc;
    }
    cudaMemset(c->d_status, 0, sizeof(uint32_t));
    *out = c;
    return OXG_OK;
}

int oxg_destroy(oxg_context* c)
{
    if (!c) return OXG_OK;
    dfree(c->d_block);
    dfree(c->d_status);
    dfree(c->conv);
    delete c;
    return OXG_OK;
}

int oxg_set_excvol_params(oxg_context* c, int ti, int tj, const oxg_excvol_params* p, double r)
{ return set_pair(c, c->excvol, ti, tj, p, r); }
int oxg_set_hbond_params(oxg_context* c, int ti, int tj, const oxg_hbond_params* p, double r)
{ return set_pair(c, c->hbond, ti, tj, p, r); }
int oxg_set_cross_params(oxg_context* c, int ti, int tj, const oxg_cross_params* p, double r)
{ return set_pair(c, c->cross, ti, tj, p, r); }
int oxg_set_hbondcross_params(oxg_context* c, int ti, int tj, const oxg_hbondcross_params* p, double r)
{ return set_pair(c, c->hbx, ti, tj, p, r); }
int oxg_set_coax_params(oxg_context* c, int ti, int tj, const oxg_coax_params* p, double r)
{ return set_pair(c, c->coax, ti, tj, p, r); }
int oxg_set_debye_params(oxg_context* c, int ti, int tj, const oxg_debye_params* p, double r)
{ return set_pair(c, c->debye, ti, tj, p, r); }

int oxg_set_bonded_params(oxg_context* c, int bt, const oxg_bonded_params* p)
{
    if (!c || !p) return set_err(OXG_ERR_INVALID_ARG, "null context or parameters");
    if (bt < 0 || bt >= c->n_bond_types) return set_err(OXG_ERR_INVALID_ARG, "invalid bond type");
    c->bonded[bt] = *p;
    c->bonded_set[bt] = true;
    c->dirty = true;
    return OXG_OK;
}

static uint32_t present_mask(const oxg_context* c)
{
    uint32_t m = 0;
    if (c->excvol.any) m |= 1u << kExcVol;
    if (c->hbond.any) m |= 1u << kHBond;
    if (c->cross.any) m |= 1u << kCross;
    if (c->hbx.any) m |= 1u << kHBCross;
    if (c->coax.any) m |= 1u << kCoax;
    if (c->debye.any) m |= 1u << kDebye;
    return m;
}

int oxg_pair_forces(oxg_context* c, uint32_t mask, int N, const double* pos_type,
                    const double* quat, const double* charge, const float box[3],
                    const uint32_t* n_neigh, const uint32_t* nlist, const uint64_t* head_list,
                    float* force, float* torque, float* virial, double* term_energy, void* stream)
{
    if (!c || N < 0 || !box) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (mask & ~present_mask(c)) return set_err(OXG_ERR_NO_PARAMS, "a requested term has no parameters");
    if (N == 0 || mask == 0) return OXG_OK;
    if (!pos_type || !quat || !n_neigh || !nlist || !head_list || !force || !torque)
        return set_err(OXG_ERR_INVALID_ARG, "null device array");
    if (!(box[0] > 0.f && box[1] > 0.f && box[2] > 0.f)) return set_err(OXG_ERR_INVALID_ARG, "bad box");
    int rc = build_block(c);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (N > c->conv_cap) {  // grows with the largest N seen (HOOMD's N is fixed per run)
        if (c->conv) {
            OXG_CUDA(cudaStreamSynchronize(s));
            dfree(c->conv);
        }
        if ((rc = dalloc(&c->conv, (size_t)3 * N))) return rc;
        c->conv_cap = N;
    }
    HoomdConvertArgs cv;
    cv.N = N;
    cv.pos = reinterpret_cast<const double4_32a*>(pos_type);
    cv.quat = reinterpret_cast<const double4_32a*>(quat);
    cv.charge = charge;
    cv.hi = c->conv;
    cv.lo = c->conv + c->conv_cap;
    cv.q = c->conv + 2 * (size_t)c->conv_cap;
    k_hoomd_convert<<<(N + 255) / 256, 256, 0, s>>>(cv);
    HoomdPairArgs a;
    a.params = c->d_block;
    a.param_bytes = c->block_bytes;
    a.mask = mask;
    a.N = N;
    a.hi = cv.hi;
    a.lo = cv.lo;
    a.q = cv.q;
    a.n_neigh = n_neigh;
    a.nlist = nlist;
    a.head_list = reinterpret_cast<const unsigned long long*>(head_list);
    a.Lf = make_float3(box[0], box[1], box[2]);
    a.invL = make_float3(1.f / box[0], 1.f / box[1], 1.f / box[2]);
    a.force = reinterpret_cast<float4*>(force);
    a.torque = reinterpret_cast<float4*>(torque);
    a.virial = virial;
    a.energy = term_energy;
    a.status = c->d_status;
    const int threads = 256;
    const int blocks = (int)(((long long)N * 32 + threads - 1) / threads);
    if (term_energy) k_pairs_hoomd<true><<<blocks, threads, c->block_bytes, s>>>(a);
    else k_pairs_hoomd<false><<<blocks, threads, c->block_bytes, s>>>(a);
    OXG_CUDA(cudaGetLastError());
    c->last_stream = s;
    return OXG_OK;
}

int oxg_bonded_forces(oxg_context* c, int N, const double* pos_type, const double* quat,
                      const float box[3], int n_bonds, const int32_t* bonds, float* force,
                      float* torque, float* virial, double* split_energy, void* stream)
{
    if (!c || N < 0 || n_bonds < 0 || !box) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (n_bonds == 0) return OXG_OK;
    if (!pos_type || !quat || !bonds || !force || !torque)
        return set_err(OXG_ERR_INVALID_ARG, "null device array");
    for (int t = 0; t < c->n_bond_types; ++t)
        if (!c->bonded_set[t]) return set_err(OXG_ERR_NO_PARAMS, "bond type without parameters");
    int rc = build_block(c);
    if (rc) return rc;
    BondDropinArgs a;
    a.params = c->d_block;
    a.param_bytes = c->block_bytes;
    a.N = N;
    a.n_bonds = n_bonds;
    a.pos = reinterpret_cast<const double4_32a*>(pos_type);
    a.quat = reinterpret_cast<const double4_32a*>(quat);
    a.bonds = bonds;
    a.L = make_double3(box[0], box[1], box[2]);
    a.invL = make_float3(1.f / box[0], 1.f / box[1], 1.f / box[2]);
    a.force = reinterpret_cast<float4*>(force);
    a.torque = reinterpret_cast<float4*>(torque);
    a.virial = virial;
    a.energy = split_energy;
    a.status = c->d_status;
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = 64;  // a thread per bond: small blocks spread a few thousand bonds over every SM
    k_bonds_dropin<<<(n_bonds + threads - 1) / threads, threads, c->block_bytes, s>>>(a);
    OXG_CUDA(cudaGetLastError());
    c->last_stream = s;
    return OXG_OK;
}

int oxg_context_status(oxg_context* c, int clear)
{
    if (!c) return set_err(OXG_ERR_INVALID_ARG, "null context");
    OXG_CUDA(cudaStreamSynchronize(c->last_stream));
    uint32_t f = 0;
    OXG_CUDA(cudaMemcpy(&f, c->d_status, sizeof(f), cudaMemcpyDeviceToHost));
    if (clear) OXG_CUDA(cudaMemset(c->d_status, 0, sizeof(uint32_t)));
    if (f & kStBadIndex) return set_err(OXG_ERR_BAD_INDEX, "a neighbour or bond index was out of range");
    return OXG_OK;
}

}  // extern "C"

// ========================================================================= system
struct oxg_system {
    oxg_context* ctx = nullptr;
    int N = 0;
    int n_bonds = 0;
    float3 L, invL;
    cudaStream_t stream = nullptr;
    // resident state
    float4 *pos = nullptr, *pos_lo = nullptr, *quat = nullptr, *vel = nullptr, *angmom = nullptr;
    float4 *accel = nullptr, *tnet = nullptr, *pos_ref = nullptr;
    float4 *force = nullptr, *torque = nullptr;
    float* charge = nullptr;
    int4* bonds = nullptr;
    int4* excl = nullptr;
    // neighbour list
    double buffer = 0.4;
    int3 nc = make_int3(1, 1, 1);
    int use_cells = 0;
    int cell_cap = 64;
    int n_cells = 1;
    uint32_t* cell_count = nullptr;
    int* cell_list = nullptr;
    int2 *pairs_short = nullptr, *pairs_long = nullptr;
    int2* queue = nullptr;  // kNQ deferred-term queues of cap_short pairs (i, j)
    long long cap_short = 0, cap_long = 0;
    float rlist2 = 0.f, rshort2 = 0.f;
    uint32_t nlist_mask = 0xffffffffu;  // term mask the current sizing was made for
    uint64_t nlist_version = ~0ull;
    DevStatus* st = nullptr;
    DevStatus* st_host = nullptr;  // pinned
    DevStatus* st_mirror = nullptr;  // its device alias (the run kernel writes the status there)
    uint32_t run_seq = 0;            // sequence number of the last run-kernel launch (never 0,
                                     // unique in the process)
    // host session (oxg_system_set_host_session): the request block (page-locked, mapped),
    // the idle time, whether a run kernel is resident and the parameter version it staged
    HostRequest* req_host = nullptr;
    HostRequest* req_dev = nullptr;
    int session_idle_us = 0;
    bool resident = false;
    uint32_t resident_version = 0;
    int64_t session_served = 0;      // host-state runs served by a resident kernel
    int64_t run_launches = 0;        // launches of the run kernel
    double* energy = nullptr;      // 9 doubles
    // integrator
    double dt = 0.003, kT = 0.1, gamma = 1.0, gamma_r = 1.0;
    uint64_t seed = 1;
    uint32_t run_mask = 0;
    int run_bonded = 1;
    bool integ_set = false;
    unsigned long long timestep = 0;
    // checkpoint of the state at the start of a graph chunk
    float4 *ck_pos = nullptr, *ck_pos_lo = nullptr, *ck_quat = nullptr, *ck_vel = nullptr,
           *ck_angmom = nullptr;
    // graph
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    uint64_t graph_key = ~0ull;
    int grid_forces = 0;
    // persistent run kernel
    GridBarrier* bar = nullptr;
    int grid_run = 0, grid_run_host = 0;
    bool lists_valid = false;  // pair lists built for the current positions' reference
    // the force / torque arrays hold the forces of the current state (a persistent run
    // ended and nothing changed since: no state, parameter, integrator or surrogate
    // change, no read-out that reused the arrays); the next run start reuses them
    bool forces_current = false;
    uint64_t forces_version = 0;  // ctx->version they were computed with
    cudaEvent_t ev_run[2] = {nullptr, nullptr};  // around each run-kernel launch
    // the surrogate's tile kernel runs beside forces B on a second stream (fork / join
    // by events, captured as graph edges)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double run_kernel_ms = 0.0;
    long long run_kernel_launches = 0, run_kernel_bodies = 0;
    bool persistent = true;
    int block_q = kBlockQ;  // phase-A per-block queue entries (OXG_BLOCK_QUEUE test hook)
    // learned surrogate of the fused HB + cross-stacking term
    const MlpDev* mlp = nullptr;
    SurrogateAudit* audit = nullptr;
    int surr_flags = 0;
    uint32_t audit_every = 0, audit_mod = 100;
    float audit_tol = 0.f;
    // stats
    long long steps_run = 0;
};

// (defined with the run path below; every system entry point ends a host session first)
extern "C" {
static int end_session(oxg_system* s);
}

namespace {

int sys_alloc_nlist(oxg_system* s)
{
    s->lists_valid = false;  // the next run must build them
    dfree(s->cell_count);
    dfree(s->cell_list);
    dfree(s->pairs_short);
    dfree(s->pairs_long);
    dfree(s->queue);
    int rc;
    if ((rc = dalloc(&s->cell_count, (size_t)2 * s->n_cells))) return rc;
    OXG_CUDA(cudaMemset(s->cell_count, 0, sizeof(uint32_t) * 2 * s->n_cells));
    if ((rc = dalloc(&s->cell_list, (size_t)s->n_cells * s->cell_cap))) return rc;
    if ((rc = dalloc(&s->pairs_short, (size_t)s->cap_short))) return rc;
    if ((rc = dalloc(&s->pairs_long, (size_t)s->cap_long))) return rc;
    if ((rc = dalloc(&s->queue, (size_t)kNQ * s->cap_short))) return rc;
    return OXG_OK;
}

// Size the cell grid and pair lists for the current parameters and mask.
int sys_setup_nlist(oxg_system* s, uint32_t mask, bool bonded_only)
{
    int rc = build_block(s->ctx);
    if (rc) return rc;
    if (s->nlist_mask == mask && s->nlist_version == s->ctx->version && s->cell_count) return OXG_OK;
    double rmax = 0.0, rshort = 0.0;
    // per-term maxima over type pairs
    auto upd = [&](bool any, const double* rc, bool is_short, int t) {
        if (!any || !((mask >> t) & 1u)) return;
        for (int k = 0; k < kMaxPairs; ++k) {
            rmax = std::max(rmax, rc[k]);
            if (is_short) rshort = std::max(rshort, rc[k]);
        }
    };
    oxg_context* c = s->ctx;
    upd(c->excvol.any, c->excvol.rcut, true, kExcVol);
    upd(c->hbond.any, c->hbond.rcut, true, kHBond);
    upd(c->cross.any, c->cross.rcut, true, kCross);
    upd(c->hbx.any, c->hbx.rcut, true, kHBCross);
    upd(c->coax.any, c->coax.rcut, true, kCoax);
    upd(c->debye.any, c->debye.rcut, false, kDebye);
    (void)bonded_only;
    const double rlist = (rmax > 0.0 ? rmax + s->buffer : 0.0);
    s->rlist2 = (float)(rlist * rlist);
    const double rsh = rshort > 0.0 ? rshort + s->buffer : 0.0;
    s->rshort2 = (float)(rsh * rsh);
    const double Ls[3] = {s->L.x, s->L.y, s->L.z};
    int n[3];
    s->use_cells = rlist > 0.0;
    for (int d = 0; d < 3; ++d) {
        n[d] = rlist > 0.0 ? (int)std::floor(Ls[d] / rlist) : 1;
        if (n[d] < 3) s->use_cells = 0;
        n[d] = std::max(1, std::min(n[d], 1024));
    }
    if (!s->use_cells) n[0] = n[1] = n[2] = 1;
    s->nc = make_int3(n[0], n[1], n[2]);
    s->n_cells = n[0] * n[1] * n[2];
    if (s->cap_short == 0) {
        s->cap_short = 32LL * s->N + 1024;
        s->cap_long = 64LL * s->N + 1024;
    }
    if ((rc = sys_alloc_nlist(s))) return rc;
    s->nlist_mask = mask;
    s->nlist_version = c->version;
    s->graph_key = ~0ull;  // capacities or sizes changed
    return OXG_OK;
}

NlistArgs nlist_args(oxg_system* s)
{
    NlistArgs a;
    a.N = s->N;
    a.pos = s->pos;
    a.pos_ref = s->pos_ref;
    a.excl = s->excl;
    a.nc = s->nc;
    a.use_cells = s->use_cells;
    a.cell_cap = s->cell_cap;
    a.n_cells = s->n_cells;
    a.cell_count = s->cell_count;
    a.cell_list = s->cell_list;
    a.L = s->L;
    a.invL = s->invL;
    a.rlist2 = s->rlist2;
    a.rshort2 = s->rshort2;
    a.pairs_short = s->pairs_short;
    a.pairs_long = s->pairs_long;
    a.cap_short = (int)std::min<long long>(s->cap_short, 0x7fffffff);
    a.cap_long = (int)std::min<long long>(s->cap_long, 0x7fffffff);
    a.st = s->st;
    return a;
}

ForceArgs force_args(oxg_system* s, uint32_t mask, int bonded)
{
    ForceArgs a;
    a.params = s->ctx->d_block;
    a.param_bytes = s->ctx->block_bytes;
    a.mask = mask;
    a.bonded = bonded && s->n_bonds > 0;
    a.block_q = s->block_q;
    a.N = s->N;
    a.n_bonds = s->n_bonds;
    a.pos = s->pos;
    a.pos_lo = s->pos_lo;
    a.quat = s->quat;
    a.charge = s->charge;
    a.bonds = s->bonds;
    a.pairs_short = s->pairs_short;
    a.pairs_long = s->pairs_long;
    a.st = s->st;
    a.st_rw = s->st;
    a.cap_short = (int)std::min<long long>(s->cap_short, 0x7fffffff);
    a.cap_long = (int)std::min<long long>(s->cap_long, 0x7fffffff);
    a.advance_step = 0;
    a.queue = s->queue;
    a.L = s->L;
    a.invL = s->invL;
    a.force = s->force;
    a.torque = s->torque;
    a.energy = s->energy;
    a.virial = nullptr;
    return a;
}

// The surrogate, if set for this use (OXG_SURROGATE_RUN / _COMPUTE), into force args.
void surrogate_args(oxg_system* s, ForceArgs& a, bool md)
{
    const int want = md ? OXG_SURROGATE_RUN : OXG_SURROGATE_COMPUTE;
    if (!s->mlp || !(s->surr_flags & want) || !((a.mask >> kHBCross) & 1u)) return;
    a.mlp = s->mlp;
    a.audit = s->audit;
    a.audit_every = md ? s->audit_every : 0u;
    a.audit_mod = s->audit_mod;
    a.audit_tol = s->audit_tol;
}

IntegArgs integ_args(oxg_system* s)
{
    IntegArgs a;
    a.N = s->N;
    a.pos = s->pos;
    a.pos_lo = s->pos_lo;
    a.quat = s->quat;
    a.vel = s->vel;
    a.angmom = s->angmom;
    a.accel = s->accel;
    a.tnet = s->tnet;
    a.pos_ref = s->pos_ref;
    a.force = s->force;
    a.torque = s->torque;
    a.st = s->st;
    a.L = s->L;
    a.invL = s->invL;
    a.dt = (float)s->dt;
    a.kT = (float)s->kT;
    a.gamma = (float)s->gamma;
    a.gamma_r = (float)s->gamma_r;
    a.half_buf2 = (float)(0.25 * s->buffer * s->buffer);
    a.inertia = make_float3(1.f, 1.f, 1.f);
    a.seed_lo = (uint32_t)s->seed;
    a.seed_hi = (uint32_t)(s->seed >> 32);
    return a;
}

int forces_grid(oxg_system* s)
{
    if (s->grid_forces == 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_forces_a<false>, 256, s->ctx->block_bytes);
        if (per_sm < 1) per_sm = 1;
        s->grid_forces = num_sms() * per_sm;
        // the surrogate kernel's shared memory exceeds the default limit (set here, outside
        // any stream capture)
        static_assert(surrogate_smem(kParamBlockMax) <= 227 * 1024, "surrogate tile exceeds a block's shared memory");
        const int smem = (int)surrogate_smem(kParamBlockMax);
        cudaFuncSetAttribute(k_surrogate<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(k_surrogate<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    }
    if (!s->side) {  // outside any stream capture, like the attributes above
        if (cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming) != cudaSuccess)
            s->side = nullptr;
    }
    return s->grid_forces;
}

// Launch nlist (if flagged) + forces on s->stream.
int launch_nlist_forces(oxg_system* s, uint32_t mask, int bonded, bool energy, bool md_step = false)
{
    const NlistArgs na = nlist_args(s);
    const int threads = 256;
    const int nb = std::max(1, (std::max(s->N, s->n_cells) + threads - 1) / threads);
    k_nlist_bin<<<nb, threads, 0, s->stream>>>(na);
    k_nlist_pairs<<<std::max(1, (s->N + 7) / 8), threads, 0, s->stream>>>(na);  // a warp per particle
    ForceArgs fa = force_args(s, mask, bonded);
    fa.advance_step = md_step ? 1 : 0;
    surrogate_args(s, fa, md_step);
    const int grid = forces_grid(s);
    if (!md_step)  // MD steps: the integrator kernels reset the queue lengths
        OXG_CUDA(cudaMemsetAsync(s->st->qcount, 0, sizeof(s->st->qcount), s->stream));
    const bool surr = fa.mlp != nullptr;
    // the surrogate's tiles on the tensor cores between the phases (two blocks per SM)
    const uint32_t surr_smem = surrogate_smem(s->ctx->block_bytes);
    const int surr_grid = 2 * num_sms();
    if (energy) k_forces_a<true><<<grid, 256, s->ctx->block_bytes, s->stream>>>(fa);
    else k_forces_a<false><<<grid, 256, s->ctx->block_bytes, s->stream>>>(fa);
    if (surr) {
        // forces B and the surrogate tiles touch different queues and add into the
        // accumulators with atomics: they run side by side
        if (!s->side) return set_err(OXG_ERR_CUDA, "could not create the side stream");  // made by forces_grid
        OXG_CUDA(cudaEventRecord(s->ev_fork, s->stream));
        OXG_CUDA(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
        if (energy) k_surrogate<true><<<surr_grid, kSurrThreads, surr_smem, s->side>>>(fa);
        else k_surrogate<false><<<surr_grid, kSurrThreads, surr_smem, s->side>>>(fa);
        OXG_CUDA(cudaEventRecord(s->ev_join, s->side));
    }
    if (energy) k_forces_b<true><<<grid, 256, s->ctx->block_bytes, s->stream>>>(fa);
    else k_forces_b<false><<<grid, 256, s->ctx->block_bytes, s->stream>>>(fa);
    if (surr) OXG_CUDA(cudaStreamWaitEvent(s->stream, s->ev_join, 0));
    OXG_CUDA(cudaGetLastError());
    return OXG_OK;
}

int set_rebuild(oxg_system* s)
{
    const uint32_t one = 1u;
    OXG_CUDA(cudaMemcpyAsync(&s->st->rebuild, &one, sizeof(one), cudaMemcpyHostToDevice, s->stream));
    return OXG_OK;
}

int read_status(oxg_system* s, DevStatus* out)
{
    OXG_CUDA(cudaMemcpyAsync(s->st_host, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    *out = *s->st_host;
    return OXG_OK;
}

int clear_flags(oxg_system* s)
{
    OXG_CUDA(cudaMemsetAsync(&s->st->flags, 0, sizeof(uint32_t), s->stream));
    return OXG_OK;
}

// Grow whatever overflowed; returns true if something grew.
int grow_for(oxg_system* s, const DevStatus& d, bool* grew)
{
    *grew = false;
    if (d.flags & kStCellOverflow) {
        s->cell_cap = std::max<int>(s->cell_cap * 2, (int)d.max_cell + 16);
        *grew = true;
    }
    if (d.flags & kStPairOverflow) {
        s->cap_short = std::max<long long>(s->cap_short * 3 / 2, (long long)d.n_short * 5 / 4 + 1024);
        s->cap_long = std::max<long long>(s->cap_long * 3 / 2, (long long)d.n_long * 5 / 4 + 1024);
        *grew = true;
    }
    if (*grew) {
        int rc = sys_alloc_nlist(s);
        if (rc) return rc;
        s->graph_key = ~0ull;
    }
    return OXG_OK;
}

}  // namespace

extern "C" {

int oxg_system_create(oxg_system** out, oxg_context* ctx, int N, const float box[3], int n_bonds,
                      const int32_t* bonds_host)
{
    if (!out || !ctx || N <= 0 || n_bonds < 0 || !box || (n_bonds > 0 && !bonds_host))
        return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (!(box[0] > 0.f && box[1] > 0.f && box[2] > 0.f)) return set_err(OXG_ERR_INVALID_ARG, "bad box");
    *out = nullptr;
    // validate bonds and build the exclusion table on the host
    std::vector<int4> excl(N, make_int4(-1, -1, -1, -1));
    std::vector<int4> bnd(std::max(1, n_bonds));
    for (int b = 0; b < n_bonds; ++b) {
        const int A = bonds_host[3 * b], B = bonds_host[3 * b + 1], t = bonds_host[3 * b + 2];
        if (A < 0 || B < 0 || A >= N || B >= N || A == B || t < 0 || t >= ctx->n_bond_types)
            return set_err(OXG_ERR_BAD_INDEX, "bond " + std::to_string(b) + " has an invalid index or type");
        bnd[b] = make_int4(A, B, t, 0);
        for (int pass = 0; pass < 2; ++pass) {
            const int x = pass ? B : A, y = pass ? A : B;
            int4& e = excl[x];
            if (e.x < 0) e.x = y;
            else if (e.y < 0) e.y = y;
            else if (e.z < 0) e.z = y;
            else if (e.w < 0) e.w = y;
            else return set_err(OXG_ERR_CAPACITY, "a particle has more than 4 bonds");
        }
    }
    oxg_system* s = new oxg_system();
    s->ctx = ctx;
    s->N = N;
    s->n_bonds = n_bonds;
    s->L = make_float3(box[0], box[1], box[2]);
    s->invL = make_float3(1.f / box[0], 1.f / box[1], 1.f / box[2]);
    int rc = OXG_OK;
    auto fail = [&](int code) {
        oxg_system_destroy(s);
        return code;
    };
    if ((rc = dalloc(&s->pos, N)) || (rc = dalloc(&s->pos_lo, N)) || (rc = dalloc(&s->ck_pos_lo, N)) ||
        (rc = dalloc(&s->quat, N)) || (rc = dalloc(&s->vel, N)) ||
        (rc = dalloc(&s->angmom, N)) || (rc = dalloc(&s->accel, N)) || (rc = dalloc(&s->tnet, N)) ||
        (rc = dalloc(&s->pos_ref, N)) || (rc = dalloc(&s->force, N)) || (rc = dalloc(&s->torque, N)) ||
        (rc = dalloc(&s->charge, N)) || (rc = dalloc(&s->bonds, std::max(1, n_bonds))) ||
        (rc = dalloc(&s->excl, N)) || (rc = dalloc(&s->st, 1)) || (rc = dalloc(&s->energy, 9)) ||
        (rc = dalloc(&s->ck_pos, N)) || (rc = dalloc(&s->ck_quat, N)) || (rc = dalloc(&s->ck_vel, N)) ||
        (rc = dalloc(&s->ck_angmom, N)) || (rc = dalloc(&s->bar, 1)) || (rc = dalloc(&s->audit, 1)))
        return fail(rc);
    cudaMemset(s->audit, 0, sizeof(SurrogateAudit));
    cudaMemset(s->bar, 0, sizeof(GridBarrier));
    if (const char* m = std::getenv("OXG_RUN_MODE")) s->persistent = std::string(m) != "graph";
    // test hook: a smaller per-block queue in phase A exercises the spill path
    if (const char* m = std::getenv("OXG_BLOCK_QUEUE")) s->block_q = std::max(0, std::min(kBlockQ, std::atoi(m)));
    if (cudaMallocHost((void**)&s->st_host, sizeof(DevStatus)) == cudaSuccess &&
        cudaHostGetDevicePointer((void**)&s->st_mirror, s->st_host, 0) != cudaSuccess) {
        cudaGetLastError();
        s->st_mirror = nullptr;
    }
    if (!s->st_host)
        return fail(set_err(OXG_ERR_CUDA, "cudaMallocHost failed"));
    std::memset(s->st_host, 0, sizeof(DevStatus));  // (page-locked memory may be recycled)
    cudaMemcpy(s->bonds, bnd.data(), sizeof(int4) * bnd.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->excl, excl.data(), sizeof(int4) * N, cudaMemcpyHostToDevice);
    cudaMemset(s->st, 0, sizeof(DevStatus));
    cudaMemset(s->energy, 0, 9 * sizeof(double));
    // defaults: unit mass, identity orientation, zero momenta, unit charge
    std::vector<float4> v(N, make_float4(0.f, 0.f, 0.f, 1.f));
    std::vector<float4> q(N, make_float4(1.f, 0.f, 0.f, 0.f));
    std::vector<float4> z(N, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> ch(N, 1.f);
    cudaMemcpy(s->vel, v.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->quat, q.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->pos, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->pos_lo, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->angmom, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->accel, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->tnet, z.data(), sizeof(float4) * N, cudaMemcpyHostToDevice);
    cudaMemcpy(s->charge, ch.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(set_err(OXG_ERR_CUDA, cudaGetErrorString(e)));
    *out = s;
    return OXG_OK;
}

int oxg_system_destroy(oxg_system* s)
{
    if (!s) return OXG_OK;
    end_session(s);
    if (s->req_host) cudaFreeHost(s->req_host);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    dfree(s->pos); dfree(s->pos_lo); dfree(s->ck_pos_lo); dfree(s->quat); dfree(s->vel); dfree(s->angmom); dfree(s->accel);
    dfree(s->tnet); dfree(s->pos_ref); dfree(s->force); dfree(s->torque); dfree(s->charge);
    dfree(s->bonds); dfree(s->excl); dfree(s->st); dfree(s->energy);
    dfree(s->cell_count); dfree(s->cell_list); dfree(s->pairs_short); dfree(s->pairs_long);
    dfree(s->queue);
    dfree(s->ck_pos); dfree(s->ck_quat); dfree(s->ck_vel); dfree(s->ck_angmom);
    dfree(s->bar);
    dfree(s->audit);
    for (int k = 0; k < 2; ++k)
        if (s->ev_run[k]) cudaEventDestroy(s->ev_run[k]);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->st_host) cudaFreeHost(s->st_host);
    delete s;
    return OXG_OK;
}

}  // extern "C"

namespace {

// Device-accessible address of page-locked, mapped host memory (cudaHostAlloc, torch's
// pin_memory), or null for any other pointer: a state copy from or to such memory runs
// as one kernel reading or writing host memory directly instead of five copies.
const void* mapped_alias(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return at.devicePointer;
}

struct StateCopy {
    const float4* src[5];
    float4* dst[5];
    int N;
};

// One thread per particle and array: the five state arrays in one launch.
__global__ void k_state_copy(StateCopy c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.N) return;
#pragma unroll
    for (int k = 0; k < 5; ++k)
        if (c.src[k]) c.dst[k][i] = c.src[k][i];
}

// The state arrays between host and device: one kernel when every host array given is
// mapped page-locked memory, else one copy per array. Synchronises.
int state_transfer(oxg_system* s, const float* const host[5], float4* const dev[5], bool to_device)
{
    StateCopy c;
    c.N = s->N;
    bool mapped = true;
    int n = 0;
    for (int k = 0; k < 5; ++k) {
        c.src[k] = nullptr;
        c.dst[k] = nullptr;
        if (!host[k]) continue;
        ++n;
        const void* alias = mapped_alias(host[k]);
        if (!alias) mapped = false;
        if (to_device) {
            c.src[k] = static_cast<const float4*>(alias);
            c.dst[k] = dev[k];
        } else {
            c.src[k] = dev[k];
            c.dst[k] = static_cast<float4*>(const_cast<void*>(alias));
        }
    }
    if (n == 0) {
        OXG_CUDA(cudaStreamSynchronize(s->stream));
        return OXG_OK;
    }
    const size_t b4 = sizeof(float4) * s->N;
    if (mapped && s->N > 0) {
        k_state_copy<<<(s->N + 255) / 256, 256, 0, s->stream>>>(c);
        OXG_CUDA(cudaGetLastError());
    } else {
        for (int k = 0; k < 5; ++k) {
            if (!host[k]) continue;
            if (to_device) OXG_CUDA(cudaMemcpyAsync(dev[k], host[k], b4, cudaMemcpyHostToDevice, s->stream));
            else OXG_CUDA(cudaMemcpyAsync(const_cast<float*>(host[k]), dev[k], b4, cudaMemcpyDeviceToHost, s->stream));
        }
    }
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    return OXG_OK;
}

}  // namespace

extern "C" {

int oxg_system_set_stream(oxg_system* s, void* stream)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    s->stream = (cudaStream_t)stream;
    s->graph_key = ~0ull;
    return OXG_OK;
}

int oxg_system_set_state(oxg_system* s, const float* pos_type, const float* pos_lo,
                         const float* quat, const float* vel, const float* angmom,
                         const float* charge)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    s->forces_current = false;  // the next run start evaluates the forces again
    const size_t b4 = sizeof(float4) * s->N;
    if (pos_type) {
        for (int i = 0; i < s->N; ++i) {
            int t;
            std::memcpy(&t, pos_type + 4 * (size_t)i + 3, sizeof(int));
            if (t < 0 || t >= s->ctx->n_types)
                return set_err(OXG_ERR_BAD_INDEX, "particle " + std::to_string(i) + " has type " +
                                                      std::to_string(t) + " outside the context's types");
        }
        if (!pos_lo) OXG_CUDA(cudaMemsetAsync(s->pos_lo, 0, b4, s->stream));
    }
    if (charge) OXG_CUDA(cudaMemcpyAsync(s->charge, charge, sizeof(float) * s->N, cudaMemcpyHostToDevice, s->stream));
    const float* const host[5] = {pos_type, pos_lo, quat, vel, angmom};
    float4* const dev[5] = {s->pos, s->pos_lo, s->quat, s->vel, s->angmom};
    return state_transfer(s, host, dev, true);
}

int oxg_system_get_state(oxg_system* s, float* pos_type, float* pos_lo, float* quat, float* vel,
                         float* angmom)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    const float* const host[5] = {pos_type, pos_lo, quat, vel, angmom};
    float4* const dev[5] = {s->pos, s->pos_lo, s->quat, s->vel, s->angmom};
    return state_transfer(s, host, dev, false);
}

int oxg_system_device_state(oxg_system* s, float** pos_type, float** pos_lo, float** quat,
                            float** vel, float** angmom, float** charge)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    s->forces_current = false;  // the caller may write the state through these pointers
    if (pos_type) *pos_type = reinterpret_cast<float*>(s->pos);
    if (pos_lo) *pos_lo = reinterpret_cast<float*>(s->pos_lo);
    if (quat) *quat = reinterpret_cast<float*>(s->quat);
    if (vel) *vel = reinterpret_cast<float*>(s->vel);
    if (angmom) *angmom = reinterpret_cast<float*>(s->angmom);
    if (charge) *charge = s->charge;
    return OXG_OK;
}

int oxg_system_set_nlist_buffer(oxg_system* s, double buffer)
{
    if (!s || !(buffer >= 0.0)) return set_err(OXG_ERR_INVALID_ARG, "bad buffer");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    s->buffer = buffer;
    s->nlist_version = ~0ull;
    return OXG_OK;
}

int oxg_system_set_timestep(oxg_system* s, uint64_t step)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    s->timestep = step;  // the next run's RNG steps continue from here
    return OXG_OK;
}

static int system_compute_impl(oxg_system* s, uint32_t mask, int bonded)
{
    s->forces_current = false;  // the read-out reuses the force and torque arrays
    int rc = sys_setup_nlist(s, mask, false);
    if (rc) return rc;
    for (int attempt = 0; attempt < 8; ++attempt) {
        OXG_CUDA(cudaMemsetAsync(s->force, 0, sizeof(float4) * s->N, s->stream));
        OXG_CUDA(cudaMemsetAsync(s->torque, 0, sizeof(float4) * s->N, s->stream));
        OXG_CUDA(cudaMemsetAsync(s->energy, 0, sizeof(double) * 9, s->stream));
        if ((rc = clear_flags(s)) || (rc = set_rebuild(s))) return rc;
        if ((rc = launch_nlist_forces(s, mask, bonded, true))) return rc;
        DevStatus d;
        if ((rc = read_status(s, &d))) return rc;
        bool grew = false;
        if ((rc = grow_for(s, d, &grew))) return rc;
        if (!grew) return OXG_OK;
    }
    return set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
}

int oxg_system_compute(oxg_system* s, uint32_t mask, int bonded, float* force, float* torque,
                       double* pair_energy, double* bonded_energy)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    if (mask & ~present_mask(s->ctx)) return set_err(OXG_ERR_NO_PARAMS, "a requested term has no parameters");
    if (bonded)
        for (int t = 0; t < s->ctx->n_bond_types; ++t)
            if (!s->ctx->bonded_set[t]) return set_err(OXG_ERR_NO_PARAMS, "bond type without parameters");
    int rc = system_compute_impl(s, mask, bonded);
    if (rc) return rc;
    const size_t b4 = sizeof(float4) * s->N;
    if (force) OXG_CUDA(cudaMemcpyAsync(force, s->force, b4, cudaMemcpyDeviceToHost, s->stream));
    if (torque) OXG_CUDA(cudaMemcpyAsync(torque, s->torque, b4, cudaMemcpyDeviceToHost, s->stream));
    double e[9];
    OXG_CUDA(cudaMemcpyAsync(e, s->energy, sizeof(e), cudaMemcpyDeviceToHost, s->stream));
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    if (pair_energy) std::memcpy(pair_energy, e, sizeof(double) * kNTerms);
    if (bonded_energy) std::memcpy(bonded_energy, e + kNTerms, sizeof(double) * 3);
    return OXG_OK;
}

int oxg_system_set_integrator(oxg_system* s, double dt, double kT, double gamma, double gamma_r,
                              uint64_t seed, uint32_t mask, int bonded)
{
    if (!s || !(dt > 0.0) || !(kT >= 0.0) || !(gamma >= 0.0) || !(gamma_r >= 0.0))
        return set_err(OXG_ERR_INVALID_ARG, "bad integrator parameters");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    if (mask & ~present_mask(s->ctx)) return set_err(OXG_ERR_NO_PARAMS, "a requested term has no parameters");
    s->dt = dt;
    s->kT = kT;
    s->gamma = gamma;
    s->gamma_r = gamma_r;
    s->seed = seed;
    s->run_mask = mask;
    s->run_bonded = bonded;
    s->integ_set = true;
    s->forces_current = false;
    s->graph_key = ~0ull;
    return OXG_OK;
}

// Step sequence of a run of n steps (velocity Verlet split as HOOMD does):
//   prepRun, step_one, n - 1 x [nlist, forces, step_two_one], nlist, forces, step_two
// where step_two_one is step two of one step fused with step one of the next.
static int enqueue_step_one(oxg_system* s)
{
    const IntegArgs ia = integ_args(s);
    k_step_one<<<(s->N + 255) / 256, 256, 0, s->stream>>>(ia);
    OXG_CUDA(cudaGetLastError());
    return OXG_OK;
}

// One step body: forces of the current positions, then step two (+ next step one).
static int enqueue_step(oxg_system* s, bool last)
{
    int rc = launch_nlist_forces(s, s->run_mask, s->run_bonded, false, true);
    if (rc) return rc;
    const IntegArgs ia = integ_args(s);
    if (last) k_step_two<<<(s->N + 255) / 256, 256, 0, s->stream>>>(ia);
    else k_step_two_one<<<(s->N + 255) / 256, 256, 0, s->stream>>>(ia);
    OXG_CUDA(cudaGetLastError());
    return OXG_OK;
}

static int build_graph(oxg_system* s, int steps)
{
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    cudaStream_t cap = s->stream;
    bool own = false;
    if (cap == nullptr) {  // the legacy stream cannot be captured
        OXG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        own = true;
    }
    forces_grid(s);  // occupancy query outside the capture
    cudaStream_t saved = s->stream;
    s->stream = cap;
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        s->stream = saved;
        if (own) cudaStreamDestroy(cap);
        return set_err(OXG_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
    }
    int rc = OXG_OK;
    for (int k = 0; k < steps && rc == OXG_OK; ++k) rc = enqueue_step(s, false);
    e = cudaStreamEndCapture(cap, &g);
    s->stream = saved;
    if (own) cudaStreamDestroy(cap);
    if (rc) return rc;
    if (e != cudaSuccess) return set_err(OXG_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_err(OXG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    s->graph_steps = steps;
    return OXG_OK;
}

static int checkpoint(oxg_system* s, bool restore)
{
    const size_t b4 = sizeof(float4) * s->N;
    if (restore) {  // the aborted chunk left partial sums in the accumulators
        OXG_CUDA(cudaMemsetAsync(s->force, 0, b4, s->stream));
        OXG_CUDA(cudaMemsetAsync(s->torque, 0, b4, s->stream));
    }
    float4* src[5] = {s->pos, s->pos_lo, s->quat, s->vel, s->angmom};
    float4* dst[5] = {s->ck_pos, s->ck_pos_lo, s->ck_quat, s->ck_vel, s->ck_angmom};
    for (int k = 0; k < 5; ++k) {
        if (restore) OXG_CUDA(cudaMemcpyAsync(src[k], dst[k], b4, cudaMemcpyDeviceToDevice, s->stream));
        else OXG_CUDA(cudaMemcpyAsync(dst[k], src[k], b4, cudaMemcpyDeviceToDevice, s->stream));
    }
    return OXG_OK;
}

// Sequence numbers of run-kernel launches and host-session requests: one counter for
// both, so that the status mirror never holds a number a later launch or request gets.
static uint32_t next_seq()
{
    static std::atomic<uint32_t> counter{0};
    uint32_t seq;
    do seq = counter.fetch_add(1u) + 1u;
    while (seq == 0u);
    return seq;
}

// The persistent run kernel: one cooperative launch of `bodies` step bodies, preceded
// by the run start (prepRun) when `prologue` (see k_run).
static int launch_run(oxg_system* s, int bodies, bool closing, int prologue = 0,
                      unsigned long long step0 = 0, bool rebuild0 = false,
                      const float4* const* hin = nullptr, float4* const* hout = nullptr, bool reuse_ok = false,
                      bool serve = false)
{
    const int block_bytes = s->ctx->block_bytes;
    RunArgs ra;
    ra.f = force_args(s, s->run_mask, s->run_bonded);  // plain evaluators only
    const bool host_io = hin || hout;
    const void* fn = host_io ? (const void*)k_run<true> : (const void*)k_run<false>;
    int& grid = host_io ? s->grid_run_host : s->grid_run;
    if (grid == 0) {
        int per_sm = 0;
        OXG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kRunThreads, block_bytes));
        if (per_sm < 1) return set_err(OXG_ERR_CUDA, "the run kernel does not fit on an SM");
        grid = num_sms() * std::min(per_sm, OXG_RUN_BLOCKS_PER_SM);
    }
    ra.n = nlist_args(s);
    ra.g = integ_args(s);
    ra.bar = s->bar;
    ra.bodies = bodies;
    ra.closing = closing ? 1 : 0;
    ra.prologue = prologue;
    ra.rebuild0 = rebuild0 ? 1u : 0u;
    ra.step0 = step0;
    ra.ck[0] = s->ck_pos;
    ra.ck[1] = s->ck_pos_lo;
    ra.ck[2] = s->ck_quat;
    ra.ck[3] = s->ck_vel;
    ra.ck[4] = s->ck_angmom;
    for (int k = 0; k < 5; ++k) {
        ra.hin[k] = hin ? hin[k] : nullptr;
        ra.hout[k] = hout ? hout[k] : nullptr;
    }
    ra.reuse_ok = reuse_ok ? 1 : 0;
    ra.st_mirror = s->st_mirror;
    // a sequence number no other launch or host-session request of the process had
    // (never 0), and the mirror's word cleared before the launch: a stale word never
    // reads as this launch's end
    const uint32_t seq = next_seq();
    s->run_seq = seq;
    ra.seq = seq;
    if (s->st_host) *reinterpret_cast<volatile uint32_t*>(&s->st_host->seq) = 0u;
    ra.req = serve ? s->req_dev : nullptr;
    ra.idle_ns = (unsigned long long)std::max(s->session_idle_us, 0) * 1000ull;
    if (serve) {  // no request pending: the kernel waits for the next sequence number
        s->req_host->quit = 0u;
        __atomic_store_n(&s->req_host->seq, 0u, __ATOMIC_RELEASE);
    }
    // the barrier word needs no reset between launches: every completed barrier adds
    // exactly 2^31 (it is cleared at allocation and after a launch that gave up)
    void* kargs[] = {&ra};
    OXG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kRunThreads), kargs, (size_t)block_bytes, s->stream));
    return OXG_OK;
}

// The end of a run-kernel launch as the host sees it: its last block stores the status,
// then the launch's sequence number, into page-locked host memory (system-scope fences
// between, and after every block's host-array writes). Spinning on that word returns a
// few microseconds before a stream synchronisation would. Gives up after 2 ms (a longer
// launch, or one that failed before its end); the caller then synchronises the stream,
// which also reports any launch error.
static bool wait_mirror(const oxg_system* s)
{
    const volatile uint32_t* seq = &s->st_host->seq;
    const auto t0 = std::chrono::steady_clock::now();
    for (long k = 1;; ++k) {
        if (*seq == s->run_seq) {
            std::atomic_thread_fence(std::memory_order_acquire);
            return true;
        }
        if ((k & 1023) == 0 && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2)) return false;
    }
}

static void copy_mirror(const oxg_system* s, DevStatus* d)
{
    const volatile uint32_t* src = reinterpret_cast<const volatile uint32_t*>(s->st_host);
    uint32_t* dst = reinterpret_cast<uint32_t*>(d);
    for (int k = 0; k < (int)(sizeof(DevStatus) / sizeof(uint32_t)); ++k) dst[k] = src[k];
}

// A host session's request to the resident run kernel: the run's parameters, then its
// sequence number (a release store). Returns true once the status mirror shows the run's
// end, false if the kernel had left (idle time out) or failed before it took the request
// (the caller then synchronises the stream and launches).
static bool post_request(oxg_system* s, int bodies, unsigned long long step0, const float4* const* hin,
                         float4* const* hout, bool reuse_ok)
{
    HostRequest* r = s->req_host;
    r->quit = 0u;
    r->bodies = bodies;
    r->reuse_ok = reuse_ok ? 1 : 0;
    r->step0 = step0;
    for (int k = 0; k < 5; ++k) {
        r->hin[k] = hin[k];
        r->hout[k] = hout[k];
    }
    const uint32_t seq = next_seq();
    s->run_seq = seq;
    __atomic_store_n(&r->seq, seq, __ATOMIC_RELEASE);
    const volatile uint32_t* done = &s->st_host->seq;
    for (long k = 1;; ++k) {
        if (*done == seq) {
            std::atomic_thread_fence(std::memory_order_acquire);
            return true;
        }
        if ((k & 1023) == 0 && cudaStreamQuery(s->stream) != cudaErrorNotReady) {
            const bool ok = *done == seq;  // it may have ended the run just before leaving
            std::atomic_thread_fence(std::memory_order_acquire);
            return ok;
        }
    }
}

// Ends a host session's resident kernel (a quit request; the kernel leaves at its next
// poll of the request word, or has left already) and waits for it. Every entry point that
// touches the system's device state, other than a served host-state run, calls this.
static int end_session(oxg_system* s)
{
    if (!s || !s->resident) return OXG_OK;
    s->resident = false;
    s->req_host->quit = 1u;
    __atomic_store_n(&s->req_host->seq, next_seq(), __ATOMIC_RELEASE);
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    return OXG_OK;
}

// A run of n steps on the persistent kernel, in launches of up to `chunk` step bodies.
// The first launch starts with prepRun (neighbour list if stale, forces, a = F/m, as
// HOOMD computes the net force at the start of every run() call) and the first step
// one, inside the kernel, so a run() call costs one launch and one synchronisation.
// Every launch starts from a checkpoint of the state (taken by the first launch
// itself) and is followed by the one host synchronisation of the chunk (the status
// read); after a neighbour-list overflow the lists grow and the chunk (with its
// prepRun, for the first) is replayed.
static int run_persistent(oxg_system* s, long nsteps, const float4* const* hin = nullptr,
                          float4* const* hout = nullptr)
{
    const int chunk = 2000;
    long done = 0;
    int retries = 0, rc;
    DevStatus d;
    if (!s->ev_run[0]) {
        OXG_CUDA(cudaEventCreate(&s->ev_run[0]));
        OXG_CUDA(cudaEventCreate(&s->ev_run[1]));
    }
    // the run start may reuse the last step's forces only for an unchanged state (from
    // host arrays: the kernel compares them with the device state and decides)
    const bool reuse = s->forces_current && s->forces_version == s->ctx->version && s->lists_valid;
    s->forces_current = false;
    while (done < nsteps) {
        const int todo = (int)std::min<long>(chunk, nsteps - done);
        const bool closing = done + todo == nsteps;
        const unsigned long long step0 = s->timestep + (unsigned long long)done;
        // the first launch checkpoints the state itself (a rebuild only if the lists are
        // new or a particle moved half the buffer since they were built)
        const bool first = done == 0;
        if (!first && (rc = checkpoint(s, false))) return rc;
        // the launch's device time (oxg_system_run_timing); host-state runs go untimed
        const bool timed = hin == nullptr;
        if (timed) OXG_CUDA(cudaEventRecord(s->ev_run[0], s->stream));
        // the host state goes in with the run start (not on a replay: the checkpoint holds
        // it) and comes back with the closing body
        const bool read_host = first && hin && retries == 0;
        const int prologue = first ? (read_host ? 3 : ((reuse && retries == 0) ? 2 : 1)) : 0;
        // a host session serves one-launch host-state runs with a resident kernel: the
        // run is posted to it when it is still there (and staged the current parameters)
        const bool serve = read_host && closing && hout && s->req_host && s->st_mirror && s->session_idle_us > 0;
        bool served = false;
        if (serve && s->resident && s->resident_version == s->ctx->version && s->lists_valid) {
            served = post_request(s, todo, step0, hin, hout, reuse);
            if (!served) {
                s->resident = false;
                OXG_CUDA(cudaStreamSynchronize(s->stream));  // (reports a failed kernel)
            }
        } else if ((rc = end_session(s))) {
            return rc;
        }
        if (served) {
            copy_mirror(s, &d);
            s->session_served += 1;
        } else {
            s->run_launches += 1;
            if ((rc = launch_run(s, todo, closing, prologue, step0, !s->lists_valid, read_host ? hin : nullptr,
                                 closing ? hout : nullptr, reuse, serve)))
                return rc;
            if (serve) {
                s->resident = true;
                s->resident_version = s->ctx->version;
            }
            if (timed) OXG_CUDA(cudaEventRecord(s->ev_run[1], s->stream));
            if (s->st_mirror) {  // the launch's last block wrote the status to host memory
                // (a timed launch waits for its end event, which the spin does not see)
                if (timed || !wait_mirror(s)) OXG_CUDA(cudaStreamSynchronize(s->stream));
                copy_mirror(s, &d);
            } else if ((rc = read_status(s, &d))) {
                return rc;
            }
        }
        // a resident kernel leaves before the host handles a failed or overflowed run
        if ((d.flags & (kStBarrierTimeout | kStNonFinite | kStBadIndex | kStCellOverflow | kStPairOverflow)) &&
            (rc = end_session(s)))
            return rc;
        float ms = 0.f;
        if (timed && cudaEventElapsedTime(&ms, s->ev_run[0], s->ev_run[1]) == cudaSuccess) {
            s->run_kernel_ms += ms;
            s->run_kernel_launches += 1;
            s->run_kernel_bodies += todo;
        }
        if (d.flags & kStBarrierTimeout) {
            cudaMemsetAsync(s->bar, 0, sizeof(GridBarrier), s->stream);
            return set_err(OXG_ERR_TIMEOUT, "a grid barrier wait of the run kernel gave up");
        }
        if (d.flags & kStNonFinite) return set_err(OXG_ERR_NONFINITE, "non-finite positions or orientations");
        if (d.flags & kStBadIndex) {
            clear_flags(s);
            return set_err(OXG_ERR_BAD_INDEX, "a particle type is outside the context's types");
        }
        if (d.flags & (kStCellOverflow | kStPairOverflow)) {
            if (++retries > 8) return set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
            bool grew = false;
            if ((rc = grow_for(s, d, &grew))) return rc;
            if ((rc = checkpoint(s, true))) return rc;
            s->lists_valid = false;  // the replayed prepRun rebuilds
            if (!first) {
                k_begin_run<<<1, 32, 0, s->stream>>>(s->st, step0, 1u);  // step, flags, rebuild, queues
                OXG_CUDA(cudaGetLastError());
            }
            continue;
        }
        done += todo;
        s->steps_run += todo;
        s->lists_valid = true;
    }
    s->timestep = d.step;
    s->forces_current = true;  // the closing body left the final state's forces
    s->forces_version = s->ctx->version;
    return OXG_OK;
}

// prepRun: fresh neighbour list, forces, a = F/m (HOOMD computes the net force at
// the start of every run() call).
static int prep_run(oxg_system* s)
{
    int rc;
    for (int attempt = 0; attempt < 8; ++attempt) {
        OXG_CUDA(cudaMemsetAsync(s->force, 0, sizeof(float4) * s->N, s->stream));
        OXG_CUDA(cudaMemsetAsync(s->torque, 0, sizeof(float4) * s->N, s->stream));
        if ((rc = clear_flags(s)) || (rc = set_rebuild(s))) return rc;
        if ((rc = launch_nlist_forces(s, s->run_mask, s->run_bonded, false))) return rc;
        DevStatus d;
        if ((rc = read_status(s, &d))) return rc;
        bool grew = false;
        if ((rc = grow_for(s, d, &grew))) return rc;
        if (!grew) break;
        if (attempt == 7) return set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
    }
    const IntegArgs ia = integ_args(s);
    k_prep_accel<<<(s->N + 255) / 256, 256, 0, s->stream>>>(ia);
    OXG_CUDA(cudaGetLastError());
    return OXG_OK;
}

// device aliases of mapped page-locked host arrays (all or none); see state_transfer
static bool mapped_state(const float* const host[5], float4* dev[5])
{
    for (int k = 0; k < 5; ++k) {
        dev[k] = static_cast<float4*>(const_cast<void*>(mapped_alias(host[k])));
        if (!dev[k]) return false;
    }
    return true;
}

int oxg_system_run(oxg_system* s, long nsteps)
{
    if (!s || nsteps < 0) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    if (!s->integ_set) return set_err(OXG_ERR_INVALID_ARG, "integrator not set");
    for (int t = 0; t < s->ctx->n_bond_types && s->run_bonded; ++t)
        if (!s->ctx->bonded_set[t]) return set_err(OXG_ERR_NO_PARAMS, "bond type without parameters");
    int rc = sys_setup_nlist(s, s->run_mask, false);
    if (rc) return rc;
    // MD steps with the surrogate take the per-step path (forces A | surrogate tiles on
    // the tensor cores | forces B | integrator, replayed from a CUDA graph)
    const bool surrogate_md = s->mlp && (s->surr_flags & OXG_SURROGATE_RUN) && ((s->run_mask >> kHBCross) & 1u);
    if (s->persistent && nsteps > 0 && !surrogate_md) {
        if ((rc = run_persistent(s, nsteps))) return rc;
        OXG_CUDA(cudaStreamSynchronize(s->stream));
        return OXG_OK;
    }
    s->forces_current = false;  // the per-step path keeps no such record
    // the RNG counter continues from the system's timestep
    OXG_CUDA(cudaMemcpyAsync(&s->st->step, &s->timestep, sizeof(unsigned long long),
                             cudaMemcpyHostToDevice, s->stream));
    if ((rc = prep_run(s))) return rc;
    if (nsteps == 0) {
        OXG_CUDA(cudaStreamSynchronize(s->stream));
        return OXG_OK;
    }
    if ((rc = enqueue_step_one(s))) return rc;
    // nsteps - 1 fused bodies in graph chunks, then the closing body with step two.
    // Chunk boundaries sit after a step one; on a list overflow the chunk is replayed
    // from its checkpoint with a forced neighbour-list rebuild.
    const long bodies = nsteps - 1;
    const int chunk = 100;
    long done = 0;
    int retries = 0;
    while (done < bodies) {
        const int todo = (int)std::min<long>(chunk, bodies - done);
        if (todo == chunk) {
            const uint64_t key = ((uint64_t)todo << 32) ^ s->ctx->version ^
                                 ((uint64_t)(uintptr_t)s->stream << 8);
            if (s->graph_key != key || !s->graph) {
                if ((rc = build_graph(s, todo))) return rc;
                s->graph_key = key;
            }
        }
        if ((rc = checkpoint(s, false))) return rc;
        DevStatus before;
        if ((rc = read_status(s, &before))) return rc;
        if (todo == chunk) {
            OXG_CUDA(cudaGraphLaunch(s->graph, s->stream));
        } else {
            for (int k = 0; k < todo && rc == OXG_OK; ++k) rc = enqueue_step(s, false);
            if (rc) return rc;
        }
        DevStatus d;
        if ((rc = read_status(s, &d))) return rc;
        if (d.flags & kStNonFinite) return set_err(OXG_ERR_NONFINITE, "non-finite positions or orientations");
        if (d.flags & kStBarrierTimeout) return set_err(OXG_ERR_TIMEOUT, "a tensor-core MMA of the surrogate did not complete");
        if (d.flags & (kStCellOverflow | kStPairOverflow)) {
            if (++retries > 8) return set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
            bool grew = false;
            if ((rc = grow_for(s, d, &grew))) return rc;
            if ((rc = checkpoint(s, true))) return rc;
            OXG_CUDA(cudaMemcpyAsync(&s->st->step, &before.step, sizeof(unsigned long long),
                                     cudaMemcpyHostToDevice, s->stream));
            if ((rc = clear_flags(s)) || (rc = set_rebuild(s))) return rc;
            s->graph_key = ~0ull;
            continue;
        }
        done += todo;
        s->steps_run += todo;
    }
    // closing body: forces at the last positions and step two
    for (int attempt = 0;; ++attempt) {
        if ((rc = checkpoint(s, false))) return rc;
        DevStatus before;
        if ((rc = read_status(s, &before))) return rc;
        if ((rc = enqueue_step(s, true))) return rc;
        DevStatus d;
        if ((rc = read_status(s, &d))) return rc;
        if (d.flags & kStNonFinite) return set_err(OXG_ERR_NONFINITE, "non-finite positions or orientations");
        if (d.flags & kStBarrierTimeout) return set_err(OXG_ERR_TIMEOUT, "a tensor-core MMA of the surrogate did not complete");
        if (!(d.flags & (kStCellOverflow | kStPairOverflow))) {
            s->timestep = d.step;
            s->steps_run += 1;
            break;
        }
        if (attempt >= 8) return set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
        bool grew = false;
        if ((rc = grow_for(s, d, &grew))) return rc;
        if ((rc = checkpoint(s, true))) return rc;
        OXG_CUDA(cudaMemcpyAsync(&s->st->step, &before.step, sizeof(unsigned long long),
                                 cudaMemcpyHostToDevice, s->stream));
        if ((rc = clear_flags(s)) || (rc = set_rebuild(s))) return rc;
    }
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    return OXG_OK;
}

int oxg_system_energies(oxg_system* s, double* pair_energy, double* bonded_energy)
{
    if (!s) return set_err(OXG_ERR_INVALID_ARG, "null system");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    uint32_t mask = s->integ_set ? s->run_mask : present_mask(s->ctx);
    int bonded = s->integ_set ? s->run_bonded : 1;
    return oxg_system_compute(s, mask, bonded, nullptr, nullptr, pair_energy, bonded_energy);
}

}  // extern "C"

namespace {

// Training samples of the surrogate: every queued fused HB + CS pair (both classes)
// gives its 7 base-base features, its class and the plain evaluator's pair energy.
__global__ void k_hbx_samples(ForceArgs a, int max_n, float* feats, float* energy, uint32_t* counter)
{
    const ParamView P = stage_params(a.params, a.param_bytes);
    const ParamHeader& H = P.h();
    const int n1 = (int)min(ld_volatile(&a.st_rw->qcount[kQHBX]), (uint32_t)a.cap_short);
    const int n0 = (int)min(ld_volatile(&a.st_rw->qcount[kQHBX0]), (uint32_t)a.cap_short);
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < n1 + n0; it += gridDim.x * blockDim.x) {
        const int q = it < n1 ? kQHBX : kQHBX0, k = it < n1 ? it : it - n1;
        PairIn p;
        bool bad = false;
        if (!load_pair(a, __ldcg(a.queue + (size_t)q * a.cap_short + k), H.n_types, p, bad)) continue;
        const Frame fi = quat_frame(p.qi), fj = quat_frame(p.qj);
        const DHBCross& px = P.term<DHBCross>(kHBCross, p.pidx);
        BBGeom g;
        if (!bb_geometry(p.rc, fi, fj, px.base, g)) continue;
        PairAcc acc;
        acc.fi = acc.ti = acc.tj = mk3(0.f, 0.f, 0.f);
        RadialF1 R1{px.f1, H.hbx_eps[p.pidx], H.hbx_shift[p.pidx]};
        float e = bb_term<false>(g, fi, fj, px.hb_t1, px.hb_t23, px.hb_t4, px.hb_t78, true, R1, acc);
        RadialF2 R2{px.f2};
        e += bb_term<true>(g, fi, fj, px.cs_t1, px.cs_t23, px.cs_t4, px.cs_t78, true, R2, acc);
        const uint32_t slot = atomicAdd(counter, 1u);
        if (slot >= (uint32_t)max_n) continue;
        float x[kMlpIn];
        mlp_features(g, x);
        for (int f = 0; f < kMlpIn; ++f) feats[(size_t)slot * 8 + f] = x[f];
        feats[(size_t)slot * 8 + 7] = q == kQHBX ? 1.f : 0.f;
        energy[slot] = e;
    }
}

}  // namespace

extern "C" {

int oxg_system_hbx_samples(oxg_system* s, int max_n, float* feats, float* energy, int* n_out)
{
    if (!s || max_n < 0 || (max_n > 0 && (!feats || !energy)) || !n_out)
        return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    if (!s->ctx->hbx.any) return set_err(OXG_ERR_NO_PARAMS, "no fused HB + cross-stacking parameters");
    s->forces_current = false;  // the sampling evaluation reuses the force arrays
    const uint32_t mask = 1u << kHBCross;
    int rc = sys_setup_nlist(s, mask | s->run_mask, false);
    if (rc) return rc;
    uint32_t* counter = nullptr;
    if ((rc = dalloc(&counter, 1))) return rc;
    for (int attempt = 0;; ++attempt) {
        OXG_CUDA(cudaMemsetAsync(counter, 0, sizeof(uint32_t), s->stream));
        if ((rc = clear_flags(s)) || (rc = set_rebuild(s))) break;
        if ((rc = launch_nlist_forces(s, mask, 0, false))) break;
        DevStatus d;
        if ((rc = read_status(s, &d))) break;
        bool grew = false;
        if ((rc = grow_for(s, d, &grew))) break;
        if (grew) {
            if (attempt == 7) {
                rc = set_err(OXG_ERR_NLIST_OVERFLOW, "neighbour list kept overflowing");
                break;
            }
            continue;
        }
        const ForceArgs fa = force_args(s, mask, 0);
        k_hbx_samples<<<2 * num_sms(), 256, s->ctx->block_bytes, s->stream>>>(fa, max_n, feats, energy, counter);
        if (cudaGetLastError() != cudaSuccess) {
            rc = set_err(OXG_ERR_CUDA, "sample kernel launch failed");
            break;
        }
        uint32_t n = 0;
        if (cudaMemcpyAsync(&n, counter, sizeof(n), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess) {
            rc = set_err(OXG_ERR_CUDA, "sample read-back failed");
            break;
        }
        *n_out = (int)std::min<uint32_t>(n, (uint32_t)max_n);
        break;
    }
    // the evaluation zeroes nothing the MD state needs, but leaves queue lengths behind
    cudaMemsetAsync(s->st->qcount, 0, sizeof(s->st->qcount), s->stream);
    cudaMemsetAsync(s->force, 0, sizeof(float4) * s->N, s->stream);
    cudaMemsetAsync(s->torque, 0, sizeof(float4) * s->N, s->stream);
    cudaStreamSynchronize(s->stream);
    dfree(counter);
    return rc;
}

int oxg_system_run_host(oxg_system* s, long nsteps, float* pos_type, float* pos_lo, float* quat, float* vel,
                        float* angmom)
{
    if (!s || nsteps < 1 || !pos_type || !pos_lo || !quat || !vel || !angmom)
        return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (!s->integ_set) return set_err(OXG_ERR_INVALID_ARG, "integrator not set");
    const float* const host[5] = {pos_type, pos_lo, quat, vel, angmom};
    float4* dev[5];
    int rc;
    // (MD steps with the surrogate take the per-step path of oxg_system_run)
    const bool surrogate_md = s->mlp && (s->surr_flags & OXG_SURROGATE_RUN) && ((s->run_mask >> kHBCross) & 1u);
    if (!s->persistent || surrogate_md || !mapped_state(host, dev)) {  // per-call transfers (types checked there)
        if ((rc = oxg_system_set_state(s, pos_type, pos_lo, quat, vel, angmom, nullptr))) return rc;
        if ((rc = oxg_system_run(s, nsteps))) return rc;
        return oxg_system_get_state(s, pos_type, pos_lo, quat, vel, angmom);
    }
    for (int t = 0; t < s->ctx->n_bond_types && s->run_bonded; ++t)
        if (!s->ctx->bonded_set[t]) return set_err(OXG_ERR_NO_PARAMS, "bond type without parameters");
    if ((rc = sys_setup_nlist(s, s->run_mask, false))) return rc;
    // the run kernel reads the mapped host arrays at its start and writes them in its
    // closing body; run_persistent synchronises after every launch
    return run_persistent(s, nsteps, dev, dev);
}

int oxg_system_set_host_session(oxg_system* s, int idle_us)
{
    if (!s || idle_us < 0 || idle_us > 100000) return set_err(OXG_ERR_INVALID_ARG, "idle time outside [0, 100000] us");
    if (int rc = end_session(s)) return rc;
    if (idle_us > 0 && !s->req_host) {
        if (cudaHostAlloc((void**)&s->req_host, sizeof(HostRequest), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void**)&s->req_dev, s->req_host, 0) != cudaSuccess) {
            cudaGetLastError();
            if (s->req_host) cudaFreeHost(s->req_host);
            s->req_host = nullptr;
            s->req_dev = nullptr;
            return set_err(OXG_ERR_CUDA, "page-locked request block for the host session");
        }
        std::memset(s->req_host, 0, sizeof(HostRequest));
    }
    s->session_idle_us = idle_us;
    return OXG_OK;
}

int oxg_system_run_timing(oxg_system* s, double* out, int n, int reset)
{
    if (!s || !out) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    const double v[3] = {s->run_kernel_ms, (double)s->run_kernel_launches, (double)s->run_kernel_bodies};
    for (int k = 0; k < n && k < 3; ++k) out[k] = v[k];
    if (reset) {
        s->run_kernel_ms = 0.0;
        s->run_kernel_launches = s->run_kernel_bodies = 0;
    }
    return OXG_OK;
}

int oxg_system_set_surrogate(oxg_system* s, const oxg_mlp* mlp, int flags, int audit_every,
                             int audit_mod, double audit_tol)
{
    if (!s || flags < 0 || flags > (OXG_SURROGATE_RUN | OXG_SURROGATE_COMPUTE) || audit_every < 0 ||
        audit_mod < 1 || !(audit_tol >= 0.0))
        return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    if (mlp && flags && !s->ctx->hbx.any)
        return set_err(OXG_ERR_NO_PARAMS, "the surrogate replaces the fused HB + cross-stacking term, which has no parameters");
    s->mlp = static_cast<const MlpDev*>(internal_mlp_device(mlp));
    s->surr_flags = mlp ? flags : 0;
    s->audit_every = (uint32_t)audit_every;
    s->audit_mod = (uint32_t)audit_mod;
    s->audit_tol = (float)audit_tol;
    s->graph_key = ~0ull;  // the captured steps launch the surrogate kernel or not
    s->forces_current = false;
    OXG_CUDA(cudaMemsetAsync(s->audit, 0, sizeof(SurrogateAudit), s->stream));
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    return OXG_OK;
}

int oxg_system_surrogate_stats(oxg_system* s, double* out, int n)
{
    if (!s || !out) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    SurrogateAudit h;
    OXG_CUDA(cudaMemcpyAsync(&h, s->audit, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    OXG_CUDA(cudaStreamSynchronize(s->stream));
    const double na = h.n_audited ? (double)h.n_audited : 1.0;
    const double mean = h.sum_de / na;
    const double rel = h.sum_e != 0.0 ? h.sum_de / h.sum_e : 0.0;
    const double rel_se =
        h.sum_e != 0.0 ? std::sqrt(std::max(h.sum_sq_de / na - mean * mean, 0.0) * na) / std::fabs(h.sum_e) : 0.0;
    const double v[11] = {(double)(h.disabled | h.pending), (double)h.n_audited, (double)h.n_over,
                          std::sqrt(h.sum_sq_de / na), std::sqrt(h.sum_sq_e / na),
                          std::sqrt(h.sum_sq_df / na), std::sqrt(h.sum_sq_f / na),
                          (double)h.max_abs_de, (double)h.max_abs_df, rel, rel_se};
    for (int k = 0; k < n && k < 11; ++k) out[k] = v[k];
    return OXG_OK;
}

int oxg_system_stats(oxg_system* s, int64_t* out, int n)
{
    if (!s || !out) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (int rc_ = end_session(s)) return rc_;  // a resident kernel leaves first
    DevStatus d;
    int rc = read_status(s, &d);
    if (rc) return rc;
    const int64_t v[7] = {s->steps_run, (int64_t)d.builds, (int64_t)d.n_short, (int64_t)d.n_long, 5,
                          s->session_served, s->run_launches};
    for (int k = 0; k < n && k < 7; ++k) out[k] = v[k];
    return OXG_OK;
}

}  // extern "C"

// =================================================================== bounded-wait self-test
namespace {
// One grid barrier of the run kernel's kind (grid_arrive / grid_wait) over the launch's
// blocks, of which block `skip_block` (none if negative) never arrives: the others then
// poll until the barrier's poll limit, the first to reach it sets the abort word, and
// all return. ok_out[b]: 1 passed the barrier, 0 gave up, -1 skipped it.
__global__ void k_barrier_selftest(GridBarrier* gb, int skip_block, int* ok_out)
{
    if ((int)blockIdx.x == skip_block) {
        if (threadIdx.x == 0) ok_out[blockIdx.x] = -1;
        return;
    }
    const uint32_t old = grid_arrive(gb);
    const bool ok = grid_wait(gb, old);
    if (threadIdx.x == 0) ok_out[blockIdx.x] = ok ? 1 : 0;
}
}  // namespace

extern "C" int oxg_selftest_barrier(int n_blocks, int skip_block, int* results, void* stream)
{
    if (n_blocks < 2 || n_blocks > 64 || skip_block >= n_blocks || !results)
        return set_err(OXG_ERR_INVALID_ARG, "n_blocks must be 2..64, skip_block < n_blocks, results non-null");
    if (n_blocks > num_sms()) return set_err(OXG_ERR_INVALID_ARG, "more blocks than SMs");
    cudaStream_t s = (cudaStream_t)stream;
    GridBarrier* gb = nullptr;
    int* d_ok = nullptr;
    int rc = dalloc(&gb, 1);
    if (!rc) rc = dalloc(&d_ok, (size_t)n_blocks);
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s);
        if (e == cudaSuccess) {
            void* kargs[] = {&gb, &skip_block, &d_ok};
            e = cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(n_blocks), dim3(32), kargs, 0, s);
        }
        GridBarrier h;
        if (e == cudaSuccess) e = cudaMemcpyAsync(results, d_ok, sizeof(int) * n_blocks, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, gb, sizeof(GridBarrier), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = set_err(OXG_ERR_CUDA, std::string("barrier self-test: ") + cudaGetErrorString(e));
        else if (h.abort) rc = set_err(OXG_ERR_TIMEOUT, "a grid barrier wait gave up (self-test)");
    }
    dfree(gb);
    dfree(d_ok);
    return rc;
}

// =================================================================== allocation-free
// oxg_pair_forces_noalloc: the system engine's nonbonded evaluation (cell list, split
// pair lists, fused force kernel) for callers that cannot allocate GPU memory. All of
// its scratch (parameter block, status, zero low-order positions, exclusions, cells,
// pair lists) lives in one file-scope device array of fixed size; every GPU that loads
// this library holds it until the process exits. The entry point calls no cudaMalloc,
// cudaFree or other allocating routine: it only copies into and launches on that array.
#include <mutex>

namespace {

constexpr int kNaMaxParticles = OXG_NOALLOC_MAX_PARTICLES;
constexpr int kNaMaxCellsDim = 20;  // larger boxes get larger (still >= r_list) cells
constexpr int kNaMaxCells = kNaMaxCellsDim * kNaMaxCellsDim * kNaMaxCellsDim;
constexpr int kNaCellCap = 64;
constexpr long long kNaShortCap = 32LL * kNaMaxParticles;
constexpr long long kNaLongCap = 48LL * kNaMaxParticles;
constexpr uint32_t kStExclOverflow = 16u;  // a particle with more than 4 bonds

constexpr size_t na_align(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNaOffParams = 0;
constexpr size_t kNaOffStatus = na_align(kNaOffParams + kParamBlockMax);
constexpr size_t kNaOffEnergy = na_align(kNaOffStatus + sizeof(DevStatus));
constexpr size_t kNaOffPosLo = na_align(kNaOffEnergy + 16 * sizeof(double));
constexpr size_t kNaOffPosRef = na_align(kNaOffPosLo + sizeof(float4) * kNaMaxParticles);
constexpr size_t kNaOffExcl = na_align(kNaOffPosRef + sizeof(float4) * kNaMaxParticles);
constexpr size_t kNaOffCellCount = na_align(kNaOffExcl + sizeof(int4) * kNaMaxParticles);
constexpr size_t kNaOffCellList = na_align(kNaOffCellCount + sizeof(uint32_t) * 2 * kNaMaxCells);
constexpr size_t kNaOffShort = na_align(kNaOffCellList + sizeof(int) * (size_t)kNaMaxCells * kNaCellCap);
constexpr size_t kNaOffLong = na_align(kNaOffShort + sizeof(int2) * kNaShortCap);
constexpr size_t kNaOffQueue = na_align(kNaOffLong + sizeof(int2) * kNaLongCap);
constexpr size_t kNaBytes = na_align(kNaOffQueue + sizeof(int2) * kNQ * kNaShortCap);  // ~18.1 MB

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {

std::mutex g_na_mutex;
void* g_na_ptr[256];  // device address of g_noalloc_scratch, per device ordinal
void* g_na_ctx[256];  // the driver context that address belongs to

// The current driver context (cuCtxGetCurrent through the runtime's entry-point query,
// so the library needs no link against the driver library); null if unavailable.
void* current_driver_context()
{
    using CtxGetCurrent = int (*)(void**);
    static CtxGetCurrent fn = []() -> CtxGetCurrent {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    void* ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Set-up, once per device with that device current: the symbol's device address. The
// address is looked up again when the device's context has changed since (after a
// cudaDeviceReset the module is loaded again, possibly at another address).
int noalloc_scratch(unsigned char** out)
{
    int dev = 0;
    OXG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return set_err(OXG_ERR_INVALID_ARG, "device ordinal out of range");
    void* const ctx = current_driver_context();  // null before the runtime's first call on this thread
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev] || !ctx || ctx != g_na_ctx[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return set_err(OXG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_na_ptr[dev] = p;
        g_na_ctx[dev] = current_driver_context();  // current now: the lookup initialised it
    }
    *out = static_cast<unsigned char*>(g_na_ptr[dev]);
    return OXG_OK;
}

// Clear everything the evaluation expects to start at zero (or empty) for this call.
__global__ void k_noalloc_prepare(int N, float4* pos_lo, int4* excl, float4* force,
                                  float4* torque, uint32_t* cell_count, int n_count,
                                  DevStatus* st, double* energy)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int c = i; c < n_count; c += gridDim.x * blockDim.x) cell_count[c] = 0u;
    if (i < N) {
        pos_lo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        excl[i] = make_int4(-1, -1, -1, -1);
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (i == 0) {
        st->flags = 0u;
        st->rebuild = 1u;
        st->gen = 0u;
        st->n_short = 0u;
        st->n_long = 0u;
        st->builds = 0u;
        st->max_cell = 0u;
        st->step = 0ull;
        for (int q = 0; q < kNQ; ++q) st->qcount[q] = 0u;
        for (int t = 0; t < 16; ++t) energy[t] = 0.0;
    }
}

// Bond exclusions from (A, B, type) triples: up to 4 partners per particle.
__global__ void k_noalloc_excl(int N, int n_bonds, const int* bonds, int4* excl, DevStatus* st)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_bonds) return;
    const int A = bonds[3 * b], B = bonds[3 * b + 1];
    if (A < 0 || B < 0 || A >= N || B >= N || A == B) {
        atomicOr(&st->flags, kStBadIndex);
        return;
    }
    for (int pass = 0; pass < 2; ++pass) {
        int* e = reinterpret_cast<int*>(excl + (pass ? B : A));
        const int other = pass ? A : B;
        // a bond listed twice (or as both (A, B) and (B, A)) takes one slot: a slot that
        // already holds the partner counts as stored
        bool stored = false;
        for (int k = 0; k < 4 && !stored; ++k) {
            const int prev = atomicCAS(e + k, -1, other);
            stored = prev == -1 || prev == other;
        }
        if (!stored) atomicOr(&st->flags, kStExclOverflow);
    }
}

}  // namespace

extern "C" int oxg_pair_forces_noalloc(oxg_context* c, uint32_t mask, int N,
                                       const float* pos_type, const float* quat,
                                       const float* charge, const float box[3], int n_bonds,
                                       const int32_t* bonds, float* force, float* torque,
                                       double* term_energy, void* stream)
{
    if (!c || !box || N < 0 || n_bonds < 0) return set_err(OXG_ERR_INVALID_ARG, "bad arguments");
    if (N > kNaMaxParticles)
        return set_err(OXG_ERR_CAPACITY, "oxg_pair_forces_noalloc: N = " + std::to_string(N) +
                                             " exceeds the fixed maximum of " +
                                             std::to_string(kNaMaxParticles) + " particles");
    if (n_bonds > 2 * kNaMaxParticles)
        return set_err(OXG_ERR_CAPACITY, "oxg_pair_forces_noalloc: more than " +
                                             std::to_string(2 * kNaMaxParticles) + " bonds");
    if (mask & ~present_mask(c)) return set_err(OXG_ERR_NO_PARAMS, "a requested term has no parameters");
    if (N == 0 || mask == 0) return OXG_OK;
    if (!pos_type || !quat || !force || !torque || (n_bonds > 0 && !bonds))
        return set_err(OXG_ERR_INVALID_ARG, "null device array");
    if (!(box[0] > 0.f && box[1] > 0.f && box[2] > 0.f)) return set_err(OXG_ERR_INVALID_ARG, "bad box");

    unsigned char* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    std::vector<unsigned char> blk;
    if ((rc = assemble_block(c, blk))) return rc;
    const ParamHeader& H = *reinterpret_cast<const ParamHeader*>(blk.data());
    cudaStream_t s = (cudaStream_t)stream;

    // neighbour-list geometry for a one-shot evaluation (no buffer)
    double rmax = 0.0, rshort = 0.0;
    auto upd = [&](bool any, const double* r, bool is_short, int t) {
        if (!any || !((mask >> t) & 1u)) return;
        for (int k = 0; k < kMaxPairs; ++k) {
            rmax = std::max(rmax, r[k]);
            if (is_short) rshort = std::max(rshort, r[k]);
        }
    };
    upd(c->excvol.any, c->excvol.rcut, true, kExcVol);
    upd(c->hbond.any, c->hbond.rcut, true, kHBond);
    upd(c->cross.any, c->cross.rcut, true, kCross);
    upd(c->hbx.any, c->hbx.rcut, true, kHBCross);
    upd(c->coax.any, c->coax.rcut, true, kCoax);
    upd(c->debye.any, c->debye.rcut, false, kDebye);
    const double rlist = rmax * (1.0 + 1e-6);
    int n[3];
    int use_cells = 1;
    for (int d = 0; d < 3; ++d) {
        n[d] = std::min(kNaMaxCellsDim, (int)std::floor(box[d] / rlist));
        if (n[d] < 3) use_cells = 0;
    }
    if (!use_cells) n[0] = n[1] = n[2] = 1;

    DevStatus* st = reinterpret_cast<DevStatus*>(scratch + kNaOffStatus);
    double* energy_scratch = reinterpret_cast<double*>(scratch + kNaOffEnergy);
    float4* pos_lo = reinterpret_cast<float4*>(scratch + kNaOffPosLo);
    uint32_t* cell_count = reinterpret_cast<uint32_t*>(scratch + kNaOffCellCount);
    const int n_cells = n[0] * n[1] * n[2];

    OXG_CUDA(cudaMemcpyAsync(scratch + kNaOffParams, blk.data(), blk.size(), cudaMemcpyHostToDevice, s));
    const int threads = 256;
    const int nb = std::max(1, (std::max(N, 2 * n_cells) + threads - 1) / threads);
    k_noalloc_prepare<<<nb, threads, 0, s>>>(N, pos_lo, reinterpret_cast<int4*>(scratch + kNaOffExcl),
                                             reinterpret_cast<float4*>(force),
                                             reinterpret_cast<float4*>(torque), cell_count,
                                             2 * n_cells, st, energy_scratch);
    if (n_bonds > 0)
        k_noalloc_excl<<<(n_bonds + threads - 1) / threads, threads, 0, s>>>(
            N, n_bonds, bonds, reinterpret_cast<int4*>(scratch + kNaOffExcl), st);
    if (term_energy) OXG_CUDA(cudaMemsetAsync(term_energy, 0, sizeof(double) * kNTerms, s));

    NlistArgs na;
    na.N = N;
    na.pos = reinterpret_cast<const float4*>(pos_type);
    na.pos_ref = reinterpret_cast<float4*>(scratch + kNaOffPosRef);
    na.excl = reinterpret_cast<const int4*>(scratch + kNaOffExcl);
    na.nc = make_int3(n[0], n[1], n[2]);
    na.use_cells = use_cells;
    na.cell_cap = kNaCellCap;
    na.n_cells = n_cells;
    na.cell_count = cell_count;
    na.cell_list = reinterpret_cast<int*>(scratch + kNaOffCellList);
    na.L = make_float3(box[0], box[1], box[2]);
    na.invL = make_float3(1.f / box[0], 1.f / box[1], 1.f / box[2]);
    na.rlist2 = (float)(rlist * rlist);
    na.rshort2 = (float)(rshort * rshort);
    na.pairs_short = reinterpret_cast<int2*>(scratch + kNaOffShort);
    na.pairs_long = reinterpret_cast<int2*>(scratch + kNaOffLong);
    na.cap_short = (int)kNaShortCap;
    na.cap_long = (int)kNaLongCap;
    na.st = st;
    k_nlist_bin<<<std::max(1, (std::max(N, n_cells) + threads - 1) / threads), threads, 0, s>>>(na);
    k_nlist_pairs<<<std::max(1, (N + 7) / 8), threads, 0, s>>>(na);  // a warp per particle

    ForceArgs fa;
    fa.params = scratch + kNaOffParams;
    fa.param_bytes = (int)blk.size();
    fa.mask = mask;
    fa.bonded = 0;
    fa.N = N;
    fa.n_bonds = 0;
    fa.pos = reinterpret_cast<const float4*>(pos_type);
    fa.pos_lo = pos_lo;
    fa.quat = reinterpret_cast<const float4*>(quat);
    fa.charge = charge;
    fa.bonds = nullptr;
    fa.pairs_short = na.pairs_short;
    fa.pairs_long = na.pairs_long;
    fa.st = st;
    fa.st_rw = st;
    fa.cap_short = na.cap_short;
    fa.cap_long = na.cap_long;
    fa.advance_step = 0;
    fa.queue = reinterpret_cast<int2*>(scratch + kNaOffQueue);
    fa.L = na.L;
    fa.invL = na.invL;
    fa.force = reinterpret_cast<float4*>(force);
    fa.torque = reinterpret_cast<float4*>(torque);
    fa.energy = term_energy ? term_energy : energy_scratch;
    fa.virial = nullptr;
    int per_sm = 0;
    OXG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_forces_a<true>, 256, (int)blk.size()));
    const int grid = num_sms() * std::max(1, per_sm);
    if (term_energy) {
        k_forces_a<true><<<grid, 256, blk.size(), s>>>(fa);
        k_forces_b<true><<<grid, 256, blk.size(), s>>>(fa);
    } else {
        k_forces_a<false><<<grid, 256, blk.size(), s>>>(fa);
        k_forces_b<false><<<grid, 256, blk.size(), s>>>(fa);
    }
    OXG_CUDA(cudaGetLastError());

    DevStatus d;
    OXG_CUDA(cudaMemcpyAsync(&d, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    OXG_CUDA(cudaStreamSynchronize(s));
    (void)H;
    if (d.flags & kStBadIndex) return set_err(OXG_ERR_BAD_INDEX, "a bond or particle type index is out of range");
    if (d.flags & kStExclOverflow) return set_err(OXG_ERR_CAPACITY, "a particle has more than 4 bonds");
    if (d.flags & kStCellOverflow)
        return set_err(OXG_ERR_CAPACITY, "a cell holds more than " + std::to_string(kNaCellCap) +
                                             " particles (fixed scratch limit)");
    if (d.flags & kStPairOverflow)
        return set_err(OXG_ERR_CAPACITY, "more neighbour pairs than the fixed scratch holds (" +
                                             std::to_string(kNaShortCap) + " short, " +
                                             std::to_string(kNaLongCap) + " long)");
    return OXG_OK;
}

// =================================================================== internal helpers
#include "oxg_internal.h"

namespace oxg {

int internal_set_error(int code, const std::string& msg) { return set_err(code, msg); }
int internal_assemble_block(const oxg_context* c, std::vector<unsigned char>& out)
{
    return assemble_block(c, out);
}
uint32_t internal_present_mask(const oxg_context* c) { return present_mask(c); }
double internal_max_rcut(const oxg_context* c, uint32_t mask, bool short_only)
{
    double r = 0.0;
    auto upd = [&](bool any, const double* rc, bool is_short, int t) {
        if (!any || !((mask >> t) & 1u) || (short_only && !is_short)) return;
        for (int k = 0; k < kMaxPairs; ++k) r = std::max(r, rc[k]);
    };
    upd(c->excvol.any, c->excvol.rcut, true, kExcVol);
    upd(c->hbond.any, c->hbond.rcut, true, kHBond);
    upd(c->cross.any, c->cross.rcut, true, kCross);
    upd(c->hbx.any, c->hbx.rcut, true, kHBCross);
    upd(c->coax.any, c->coax.rcut, true, kCoax);
    upd(c->debye.any, c->debye.rcut, false, kDebye);
    return r;
}
int internal_n_types(const oxg_context* c) { return c->n_types; }
bool internal_bonded_complete(const oxg_context* c)
{
    for (int t = 0; t < c->n_bond_types; ++t)
        if (!c->bonded_set[t]) return false;
    return true;
}
int internal_num_sms() { return num_sms(); }

}  // namespace oxg
