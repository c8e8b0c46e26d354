// Level internals shared by the single-level driver (level.cu) and the AMR
// hierarchy (amr.cu): FAB geometry, copy / boundary tags, the step state and
// the level object itself.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <vector>

#include "ocfd_internal.h"
#include "rhs_regular.h"

namespace ocfd {

constexpr int NGR = OCFD_NUM_GROW;
// Ghost layers the level and hierarchy fill: the regular stencils read 3 (WENO-Z
// +-3, the viscous ring +-1, coarse-fine interpolation and tagging +-1); the 4th
// layer of the NUM_GROW-wide FABs is left untouched.
constexpr int NFILL = 3;

struct FabGeom {
    int lo[3], hi[3];  // valid box
    long long off;     // element offset of the FAB in a state buffer
    int g[3];          // grown extents
    long long ns;      // component stride
};

struct ExTag {
    int dst, src;
    int lo[3], hi[3];  // region, absolute cell indices of the destination
    int shift[3];      // src cell = dst cell + shift
};

struct BcTag {
    int box, side;
    int lo[3], hi[3];
};

struct StepState {
    double time, dt, dt_prev, cfl;
    unsigned long long cfl_min;
    double stop_time;  // the last step is shortened to land on it (Source/EBR.cpp:279-286)
};

struct BcInfo {
    int lo_bc[3], hi_bc[3];
    int dom_lo[3], dom_hi[3];
    double dx[3], prob_lo[3];
    int bc_case;
    double params[16];
};

__device__ __forceinline__ long long fab_index(const FabGeom& f, int i, int j, int k) {
    return f.off + (long long)(i - f.lo[0] + NGR) + (long long)(j - f.lo[1] + NGR) * f.g[0] +
           (long long)(k - f.lo[2] + NGR) * f.g[0] * f.g[1];
}

template <class Tag>
__device__ __forceinline__ int find_tag(const long long* start, int ntag, long long idx) {
    int lo = 0, hi = ntag - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= idx) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The same through a chunk table: chunk[c] = the tag holding item c << TAG_CHUNK_LOG2,
// then a short forward scan (nullptr: the binary search)
constexpr int TAG_CHUNK_LOG2 = 7;
__device__ __forceinline__ int find_tag_chunked(const long long* start, const int* chunk, int ntag, long long idx) {
    if (!chunk) return find_tag<int>(start, ntag, idx);
    int t = chunk[idx >> TAG_CHUNK_LOG2];
    while (t + 1 < ntag && start[t + 1] <= idx) ++t;
    return t;
}

__device__ __forceinline__ void region_cell(const int* lo, const int* hi, long long local, int& i,
                                            int& j, int& k) {
    const long long nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1;
    i = lo[0] + (int)(local % nx);
    j = lo[1] + (int)((local / nx) % ny);
    k = lo[2] + (int)(local / (nx * ny));
}

// Device memory of an AMR hierarchy: released blocks are kept and handed out
// again by capacity, so regridding neither allocates nor frees in steady state
// (cudaMalloc / cudaFree synchronize the device).  Blocks are reused only after
// the caller has synchronized the work that used them.
struct DevPool {
    struct Blk {
        void* p;
        size_t cap;
    };
    std::vector<Blk> free_list;
    std::map<void*, size_t> live;
    ~DevPool() { release_all(); }
    void* get(size_t bytes) {
        bytes = std::max<size_t>(256, (bytes + 255) & ~size_t(255));
        int best = -1;
        for (int i = 0; i < (int)free_list.size(); ++i) {
            const size_t c = free_list[i].cap;
            if (c >= bytes && c <= 2 * bytes + 65536 && (best < 0 || c < free_list[best].cap)) best = i;
        }
        void* p = nullptr;
        size_t cap = bytes;
        if (best >= 0) {
            p = free_list[best].p;
            cap = free_list[best].cap;
            free_list.erase(free_list.begin() + best);
        } else {
            if (bytes >= (size_t(1) << 20)) cap = bytes + bytes / 8;  // room for a slightly larger level
            if (cudaMalloc(&p, cap) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
        }
        live[p] = cap;
        return p;
    }
    void put(void* p) {
        if (!p) return;
        auto it = live.find(p);
        if (it == live.end()) return;
        free_list.push_back({p, it->second});
        live.erase(it);
    }
    void release_all() {
        for (auto& b : free_list) cudaFree(b.p);
        for (auto& kv : live) cudaFree(kv.first);
        free_list.clear();
        live.clear();
    }
};

inline void* dev_alloc(size_t bytes, DevPool* pool) {
    if (pool) return pool->get(bytes);
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(1, bytes)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
inline void dev_free(void* p, DevPool* pool) {
    if (pool) pool->put(p);
    else cudaFree(p);
}

// ---- host helpers (level.cu)
template <class T>
ocfd_status upload(T** dptr, const std::vector<T>& v, DevPool* pool = nullptr) {
    size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
    *dptr = static_cast<T*>(dev_alloc(bytes, pool));
    if (!*dptr) return fail(OCFD_OUT_OF_MEMORY, "level table allocation");
    if (!v.empty() && cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(OCFD_LAUNCH_FAIL, "level table upload");
    return OCFD_OK;
}

bool intersect(const int* alo, const int* ahi, const int* blo, const int* bhi, int* lo, int* hi);
long long region_cells(const int* lo, const int* hi);
int grid_for(long long total, int threads, int sms);

template <class Tag>
ocfd_status upload_tags(const std::vector<Tag>& tags, Tag** d_tags, long long** d_start, long long* total,
                        DevPool* pool = nullptr, int** d_chunk = nullptr) {
    std::vector<long long> start(tags.size());
    long long acc = 0;
    for (size_t i = 0; i < tags.size(); ++i) {
        start[i] = acc;
        acc += region_cells(tags[i].lo, tags[i].hi);
    }
    *total = acc;
    ocfd_status s = upload(d_tags, tags, pool);
    if (s != OCFD_OK) return s;
    s = upload(d_start, start, pool);
    if (s != OCFD_OK || !d_chunk) return s;
    // chunk table of find_tag_chunked
    std::vector<int> chunk((size_t)((acc >> TAG_CHUNK_LOG2) + 1), 0);
    int t = 0;
    for (size_t c = 0; c < chunk.size(); ++c) {
        const long long idx = (long long)c << TAG_CHUNK_LOG2;
        while (t + 1 < (int)start.size() && start[t + 1] <= idx) ++t;
        chunk[c] = t;
    }
    return upload(d_chunk, chunk, pool);
}

struct EbLevel;
struct StageRoles;

// Time integration of a level (ebr.time_integration, Source/EBR.cpp:36 and
// Source/Advance.cpp:115-149).  Stage k reads buffer src[k], its ghosts filled at
// t + tfrac[k] dt, and writes U_out = a[k] U^n + b[k] (S + dt L(S)) into buffer
// out[k] (RK_OUT: the step's output buffer, StageRoles::out3); its face fluxes
// enter the flux registers with weight w[k] dt.  Forward Euler writes B and the
// step then copies B to the output buffer (a stage never writes the buffer it
// reads with halos).
constexpr int RK_OUT = -1;
struct RkScheme {
    int order, nst;
    int src[3], out[3];
    double a[3], b[3], tfrac[3], w[3];
    bool copy_out;
};
const RkScheme& rk_scheme(int order);

// Stage-table slots of a level: 0..nst-1 the scheme's stages, STAGE_PROBE the
// slot the autotuner and the stage timer launch (RK3's second stage, B -> C with
// U^n from A: it overwrites scratch only, whatever the scheme).
constexpr int NUM_STAGE_SLOTS = 4;
constexpr int STAGE_PROBE = 3;
struct StageSlot {
    bool used;
    int src, out;       // buffer indices
    double a, b, w;     // U^n weight, stage weight, flux-register weight (x dt)
    bool cfl;           // fused CFL bound of the new state
};
StageSlot stage_slot(int order, const StageRoles& roles, int k);

}  // namespace ocfd

struct ocfd_level {
    ocfd_context* ctx = nullptr;
    ocfd_level_desc desc{};
    std::vector<ocfd_box> boxes;
    std::vector<ocfd::FabGeom> fabs;
    long long elems = 0;      // per state buffer
    int ncomp = 5;
    // A (U^n), B, C: RK stage states; D: end-of-step state of a level that has
    // a finer level (U^n stays in A while the finer level interpolates in time)
    int nbuf = 3;
    double* buf[4] = {nullptr, nullptr, nullptr, nullptr};
    ocfd::FabGeom* d_fabs = nullptr;
    long long* d_cell_start = nullptr;
    long long ncells = 0;
    // exchange
    ocfd::ExTag* d_ex = nullptr;
    long long* d_ex_start = nullptr;
    int* d_ex_chunk = nullptr;
    int nex = 0;
    long long ex_total = 0;
    // physical BC passes
    ocfd::BcTag* d_bc[3] = {nullptr, nullptr, nullptr};
    long long* d_bc_start[3] = {nullptr, nullptr, nullptr};
    int* d_bc_chunk[3] = {nullptr, nullptr, nullptr};
    int nbc[3] = {0, 0, 0};
    long long bc_total[3] = {0, 0, 0};
    ocfd::BcInfo bcinfo{};
    // time integration order (3: SSP-RK3, 2: Heun, 1: forward Euler) and the RHS
    // stage tables, one per stage slot (ocfd::stage_slot)
    int rk_order = 3;
    int tile = 0;
    ocfd::RegBoxArgs* d_stage[ocfd::NUM_STAGE_SLOTS] = {nullptr, nullptr, nullptr, nullptr};
    int* d_tile_start = nullptr;
    int ntiles = 0;
    int nreg = 0;  // boxes in the regular stage tables
    // host copies of the regular stage tables and tiles per box (per-box launches)
    std::vector<ocfd::RegBoxArgs> h_stage[ocfd::NUM_STAGE_SLOTS];
    std::vector<int> h_ntiles;
    // tile schedule of the batched launch (TileSched) and its work-queue words
    int sched = ocfd::SCHED_GRID;
    unsigned* d_queue = nullptr;
    // the stage roles the tables were last built with (the autotuner rebuilds them)
    ocfd::StageRoles* roles = nullptr;
    ocfd::StepState* d_step = nullptr;
    bool need_estdt = true;
    // z faces with source-cell BCs on both sides: stepping leaves their outside
    // ghosts unfilled and the stencils map the loads (RegBoxArgs::zvirt)
    bool zvirt = false;
    bool zvirt_allowed = false;  // the BCs allow it (the cut-cell stencils do not)
    int zmirror[2] = {0, 0}, zsign[2] = {0, 0};
    // staging of the valid-cell copies from / to host memory (ncells x ncomp
    // doubles, allocated on first use)
    double* d_valid = nullptr;
    // device memory source: nullptr = cudaMalloc / cudaFree (standalone level),
    // else the owning hierarchy's pool (state buffers are then not zeroed)
    ocfd::DevPool* pool = nullptr;
    // embedded body: geometry, box classes, cut-cell stage tables (eb_level.cu);
    // nullptr: every box regular
    ocfd::EbLevel* eb = nullptr;
    // graph
    cudaGraphExec_t graph = nullptr;
    unsigned graph_flags = ~0u;
    double graph_cfl = -1;
};

namespace ocfd {

// Per-stage roles of a level inside an AMR hierarchy (defaults: single level).
struct StageRoles {
    int out3 = 0;              // the step's output buffer: 0 (in place over U^n) or 3
    bool cfl = true;           // fused CFL bound in the last stage
    // per box: flux-register accumulation flags and views (empty: none)
    std::vector<int> flux_bits;
    std::vector<View<double>> creg;   // 3 per box (FLUX_ACC_ALL)
    std::vector<View<double>> fplane; // 6 per box (FLUX_ACC_PLANES), [d][side]
};

ocfd_status build_stage_tables(ocfd_level* L, const StageRoles& roles);
// Ghost layers box b needs filled: NFILL for a regular box (WENO-Z +-3), 2 for a
// cut box (its primitives span grow(bx, 2)), 1 for a covered box (tagging and
// the coarse-fine slopes read +-1 around valid cells)
int box_nfill(const ocfd_level* L, int b);
// rebuild the exchange and physical-BC tables (after the box classes changed)
ocfd_status rebuild_fill_tags(ocfd_level* L);
// time every tile shape x schedule of the level's batched stage kernel, keep the
// fastest (stage tables rebuilt with the level's last roles); synchronous
ocfd_status level_autotune(ocfd_level* L, unsigned flags, int reps, cudaStream_t st);
// fill_physbc skips the z pass of a level with zvirt unless `all`
ocfd_status fill_ghosts(ocfd_level* L, double* U, double tfrac, cudaStream_t st, bool all = false);
ocfd_status fill_exchange(ocfd_level* L, double* U, cudaStream_t st);
ocfd_status fill_physbc(ocfd_level* L, double* U, double tfrac, cudaStream_t st, bool all = false);
ocfd_status launch_stage(ocfd_level* L, int s, unsigned flags, cudaStream_t st);
// kernels one launch_stage call issues
int stage_launches(const ocfd_level* L, unsigned flags);
ocfd_status launch_estdt(ocfd_level* L, cudaStream_t st);
// the valid cells of state A <-> buf (host or device; box after box, (ncomp, nz,
// ny, nx) each); in = true writes the level
ocfd_status level_copy_valid(ocfd_level* L, double* buf, bool in, cudaStream_t st);
ocfd_status level_alloc(ocfd_context* ctx, const ocfd_level_desc* desc, int nbuf, ocfd_level** out,
                        DevPool* pool = nullptr, int ncomp = 5);
__global__ void k_set_time(StepState* st, double t);
__global__ void k_reset_cfl(StepState* st);

}  // namespace ocfd
