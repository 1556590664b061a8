// C ABI of liblbm_gb300.so (declared in include/lbm_gb300.h).
//
// A handle owns one device-resident lattice: the two population buffers
// (ping-pong, structure of arrays), the class bytes, the compact boundary
// list with its per-link masks, the next-to-wall accumulators and one CUDA
// stream.  A step is one fused launch (step_kernels.cuh); batches of steps
// can be replayed from a captured CUDA graph.  Host memory is only touched by
// the explicit copy-in / read-out calls.
//
// State model.  A "start" (f = w, warm start, set_distributions or a loaded
// checkpoint) writes f^N at each point's own index into buf[0] and runs the
// prologue launch, which collides it into buf[1] (cur = 1).  Each step reads
// buf[cur] and writes buf[1-cur].  A read-out pulls from buf[1-cur] -- the
// previous step's populations -- and applies the boundary rules again, or
// reads buf[0] directly if no step ran since the start.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "lbm_internal.cuh"
#include "setup.cuh"

using namespace lbm;

struct lbm_handle {
    lbm_desc d{};
    cudaStream_t st = nullptr;
    // asynchronous outputs: device-to-host copies on a stream of their own,
    // ordered against the step stream by events
    cudaStream_t cst = nullptr;
    cudaEvent_t ev_ready = nullptr;                 // read-out launches done (step stream)
    cudaEvent_t ev_copied[2] = {nullptr, nullptr};  // copies out of the staging buffers done: macro, wss
    cudaEvent_t ev_table = nullptr;                 // last stream-ordered inlet-table upload done
    double* amp_pinned = nullptr;                   // pinned staging of that upload
    int64_t amp_pinned_cap = 0;
    std::vector<int64_t> wave_off_h, wave_len_h;    // layout of the uploaded waveforms
    std::string err;
    int nx = 0, ny = 0, nz = 0;
    int64_t npts = 0, stride = 0;
    int32_t* seg_delta = nullptr;  // per pull segment: Q offsets in active-index space
    int64_t nseg = 0;
    int32_t* seg_abs = nullptr;      // compact step kernel: rows of q * stride + delta_q
    uint32_t* warp_block = nullptr;  // compact step kernel: a block of words per warp of 32 active nodes
    GeometryLists g;
    bool has_geo = false;
    bool has_state = false;
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    void* stale = nullptr;
    void* nw_prev = nullptr;
    double *nw_n = nullptr, *nw_wss = nullptr, *nw_acc = nullptr, *nw_accm = nullptr;
    float *nw_nf = nullptr, *nw_wssf = nullptr;  // FP32-arithmetic formats
    int64_t nw_stride = 0;                         // plane stride of nw_nf
    int32_t* tile_plan = nullptr;                  // tiled step kernel (physics, FP32-arithmetic formats)
    float* sp_q = nullptr;                         // interpolated bounce-back: wall distances [Q][nsp]
    TileGeom tile{};
    float* nw_ring = nullptr;                      // float4 [kRingSlots][nnw]
    double* nw_out = nullptr;                      // read-out staging, [5][nnw]
    double* nw_fields = nullptr;                   // lbm_get_wss outputs, assembled on the device
    float2* nw_accf = nullptr;
    bool wss_from_ckpt = false;  // |tau| of the last step comes from a checkpoint (nw_wssf), not the ring
    // inlet waveforms: host tables, device concatenation with per-wave offset / length
    std::vector<std::vector<double>> waves;
    double* amp = nullptr;
    int64_t amp_cap = 0;
    int64_t* wave_off = nullptr;  // [LBM_MAX_WAVES]
    int64_t* wave_len = nullptr;  // [LBM_MAX_WAVES]
    int64_t* slots = nullptr;   // step counter, two slots (even / odd launches)
    int64_t steps = 0;          // steps taken
    int64_t since_start = 0;    // steps since the last start
    unsigned* flags = nullptr;
    std::vector<BCDev> bc;          // boundary-condition rules (host copy)
    BCDev* bct = nullptr;           // the same on the device
    std::vector<int32_t> sp_bc;     // rule of each boundary-list entry (host copy)
    double* sp_flux = nullptr;      // read-out: per-entry flux
    int nbc = 0;
    int64_t launches = 0;
    int64_t nblocks = 0;
    double* partials = nullptr;
    double* sums = nullptr;
    double* out_f = nullptr;    // read-out scratch, allocated on first use
    double* macro = nullptr;    // rho / u read-out scratch
    int graph_steps = 0;
    int persist = 0;             // steps per persistent launch (0: one launch per step)
    unsigned* bar = nullptr;     // grid barrier of persistent launches: arrivals, extra arrivals (tests)
    cudaGraphExec_t gexec = nullptr;
    int gexec_parity = -1;
    int gexec_cur = -1;
    int variant = 0;            // launch shape of the step kernel (lbm_autotune)
    size_t geo_bytes = 0;
    lbm_counts counts{};
};

namespace {

thread_local std::string g_err;

const char* code_name(int code) {
    switch (code) {
        case LBM_ERR_ARG: return "invalid argument";
        case LBM_ERR_CUDA: return "CUDA error";
        case LBM_ERR_STATE: return "bad call order";
        case LBM_ERR_NONFINITE: return "non-finite state";
        case LBM_ERR_ALLOC: return "allocation failed";
        case LBM_ERR_IO: return "I/O error";
        case LBM_ERR_UNSUPPORTED: return "unsupported";
        default: return "error";
    }
}

int fail(lbm_handle* h, int code, const std::string& msg) {
    std::string m = std::string(code_name(code)) + ": " + msg;
    if (h) h->err = m;
    else g_err = m;
    return code;
}

#define CK(h, call)                                                                          \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(h, _e == cudaErrorMemoryAllocation ? LBM_ERR_ALLOC : LBM_ERR_CUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(_e));                 \
    } while (0)

#define REQUIRE(h, cond, code, msg) \
    do {                            \
        if (!(cond)) return fail(h, code, msg); \
    } while (0)

int elem_size(int precision) {
    switch (precision) {
        case LBM_F64: return 8;
        case LBM_F32: return 4;
        case LBM_F16:
        case LBM_BF16: return 2;
        default: return 0;
    }
}

size_t real_size(int precision) { return precision == LBM_F64 ? 8 : 4; }

template <typename T>
cudaError_t dalloc(lbm_handle* h, T** p, size_t bytes) {
    bytes = bytes ? bytes : 16;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), bytes);
    if (e == cudaSuccess) h->geo_bytes += bytes;
    return e;
}

void drop_graph(lbm_handle* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gexec_parity = -1;
}

// Concatenate the host waveforms into the device table; unset waveforms
// have length 0 (amplitude 0).
int upload_waves(lbm_handle* h) {
    std::vector<int64_t> off(LBM_MAX_WAVES, 0), len(LBM_MAX_WAVES, 0);
    int64_t total = 0;
    for (size_t w = 0; w < h->waves.size(); ++w) {
        off[w] = total;
        len[w] = (int64_t)h->waves[w].size();
        total += len[w];
    }
    if (total <= h->amp_cap && off == h->wave_off_h && len == h->wave_len_h) {
        // same layout: a stream-ordered copy through pinned staging, with no
        // host wait -- steps already enqueued read the old table, later
        // steps the new one
        if (total > h->amp_pinned_cap) {
            if (h->ev_table) CK(h, cudaEventSynchronize(h->ev_table));
            if (h->amp_pinned) cudaFreeHost(h->amp_pinned);
            h->amp_pinned = nullptr;
            h->amp_pinned_cap = 0;
            CK(h, cudaHostAlloc(&h->amp_pinned, sizeof(double) * total, cudaHostAllocDefault));
            h->amp_pinned_cap = total;
        }
        if (!h->ev_table) CK(h, cudaEventCreateWithFlags(&h->ev_table, cudaEventDisableTiming));
        else CK(h, cudaEventSynchronize(h->ev_table));  // the staging's previous copy has run
        for (size_t w = 0; w < h->waves.size(); ++w)
            if (len[w] > 0) std::memcpy(h->amp_pinned + off[w], h->waves[w].data(), sizeof(double) * len[w]);
        if (total > 0)
            CK(h, cudaMemcpyAsync(h->amp, h->amp_pinned, sizeof(double) * total, cudaMemcpyHostToDevice, h->st));
        CK(h, cudaEventRecord(h->ev_table, h->st));
        return LBM_OK;
    }
    CK(h, cudaStreamSynchronize(h->st));
    if (total > h->amp_cap) {
        drop_graph(h);  // the table pointer is baked into captured launches
        if (h->amp) cudaFree(h->amp);
        h->amp = nullptr;
        h->amp_cap = 0;
        CK(h, cudaMalloc(&h->amp, sizeof(double) * total));
        h->amp_cap = total;
    }
    for (size_t w = 0; w < h->waves.size(); ++w)
        if (len[w] > 0)
            CK(h, cudaMemcpyAsync(h->amp + off[w], h->waves[w].data(), sizeof(double) * len[w],
                                  cudaMemcpyHostToDevice, h->st));
    CK(h, cudaMemcpyAsync(h->wave_off, off.data(), sizeof(int64_t) * LBM_MAX_WAVES, cudaMemcpyHostToDevice, h->st));
    CK(h, cudaMemcpyAsync(h->wave_len, len.data(), sizeof(int64_t) * LBM_MAX_WAVES, cudaMemcpyHostToDevice, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    h->wave_off_h = off;
    h->wave_len_h = len;
    return LBM_OK;
}

// The copy stream and its events (created on first use).
int ensure_copy_stream(lbm_handle* h) {
    if (h->cst) return LBM_OK;
    CK(h, cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking));
    CK(h, cudaEventCreateWithFlags(&h->ev_ready, cudaEventDisableTiming));
    CK(h, cudaEventCreateWithFlags(&h->ev_copied[0], cudaEventDisableTiming));
    CK(h, cudaEventCreateWithFlags(&h->ev_copied[1], cudaEventDisableTiming));
    // nothing pending yet: record both on the empty copy stream
    CK(h, cudaEventRecord(h->ev_copied[0], h->cst));
    CK(h, cudaEventRecord(h->ev_copied[1], h->cst));
    return LBM_OK;
}

// A read-out about to overwrite staging buffer `which` (0 macro, 1 wss)
// waits, on the step stream, for the copies still reading it.
int wait_staging(lbm_handle* h, int which) {
    if (h->cst) CK(h, cudaStreamWaitEvent(h->st, h->ev_copied[which], 0));
    return LBM_OK;
}

void free_geometry(lbm_handle* h) {
    if (h->cst) cudaStreamSynchronize(h->cst);  // copies still reading staging buffers
    GeometryLists& g = h->g;
    void* ptrs[] = {g.cls, g.sp_pt, g.sp_miss, g.sp_cls, g.sp_nw, g.sp_bc, g.bcidx, g.sp_prof, g.nw_pt, g.act_word,
                    g.sp_of_act, h->bct, h->sp_flux,
                    g.act_idx, g.act_pt,
                    h->buf[0], h->buf[1], h->stale, h->nw_prev, h->nw_n, h->nw_wss, h->nw_acc, h->nw_accm,
                    h->partials, h->sums, h->out_f, h->macro, h->seg_delta, h->nw_nf, h->nw_wssf, h->nw_accf, h->tile_plan,
                    h->nw_ring, h->nw_out, h->sp_q, h->nw_fields, h->seg_abs, h->warp_block};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    g = GeometryLists();
    h->buf[0] = h->buf[1] = h->stale = h->nw_prev = nullptr;
    h->nw_n = h->nw_wss = h->nw_acc = h->nw_accm = h->partials = h->sums = h->out_f = h->macro = nullptr;
    h->seg_delta = nullptr;
    h->nseg = 0;
    h->seg_abs = nullptr;
    h->warp_block = nullptr;
    h->bct = nullptr;
    h->sp_flux = nullptr;
    h->nw_nf = h->nw_wssf = nullptr;
    h->tile_plan = nullptr;
    h->tile = TileGeom{};
    h->sp_q = nullptr;
    h->nw_accf = nullptr;
    h->nw_ring = nullptr;
    h->nw_out = nullptr;
    h->nw_fields = nullptr;
    drop_graph(h);
    h->has_geo = h->has_state = false;
    h->geo_bytes = 0;
}

StepParams make_params(lbm_handle* h, int kind) {
    StepParams p{};
    const int parity = (int)(h->steps & 1);
    if (kind == 0) {
        p.fin = h->buf[h->cur];
        p.fout = h->buf[1 - h->cur];
    } else if (kind == 1) {
        p.fin = h->buf[0];
        p.fout = h->buf[1];
    } else {
        p.fin = h->since_start == 0 ? h->buf[0] : h->buf[1 - h->cur];
        p.direct = h->since_start == 0 ? 1 : 0;
    }
    p.stride = h->stride;
    p.seg_delta = h->seg_delta;
    p.seg_abs = h->seg_abs;
    p.warp_block = h->warp_block;
    p.nseg = h->nseg;
    p.nact = h->g.nact;
    p.act_word = h->g.act_word;
    p.sp_of_act = h->g.sp_of_act;
    p.nsp = h->g.nsp;
    p.sp_miss = h->g.sp_miss;
    p.sp_cls = h->g.sp_cls;
    p.sp_nw = h->g.sp_nw;
    p.sp_prof = h->g.sp_prof;
    p.stale = h->stale;
    p.nnw = h->g.nnw;
    p.nw_n = h->nw_n;
    p.nw_wss = h->nw_wss;
    p.nw_acc = h->nw_acc;
    p.nw_accm = h->nw_accm;
    p.nw_nf = h->nw_nf;
    p.nw_stride = h->nw_stride;
    p.tile_plan = h->tile_plan;
    p.tile = h->tile;
    p.nw_ring = h->nw_ring;
    p.nw_accf = h->nw_accf;
    p.nw_prev = h->nw_prev;
    p.tau = h->d.tau;
    p.collision = h->d.mode == LBM_PHYSICS ? h->d.collision : LBM_COLLISION_BGK;
    p.wss_C = h->d.wss_scale;
    p.inv_tau = 1.0 / h->d.tau;
    p.inv_tau_f = (float)p.inv_tau;
    p.wss_C_f = (float)h->d.wss_scale;
    p.wss_phys = -(1.0 - 0.5 / h->d.tau) * h->d.wss_scale;
    p.wss_phys_f = (float)p.wss_phys;
    p.amp = h->amp;
    p.wave_off = h->wave_off;
    p.wave_len = h->wave_len;
    p.step_base = h->slots + parity;
    p.step_next = h->slots + (1 - parity);
    p.step_off = kind == 2 ? -1 : 0;
    p.bct = h->bct;
    p.nbc = h->nbc;
    p.sp_bc = h->g.sp_bc;
    p.sp_flux = h->sp_flux;
    p.sp_q = h->d.mode == LBM_PHYSICS ? h->sp_q : nullptr;
    p.flags = h->flags;
    p.act_idx = h->g.act_idx;
    p.partials = h->partials;
    return p;
}

cudaError_t launch(lbm_handle* h, int kind, const StepParams& p) {
    h->launches++;
    switch (h->d.precision) {
        case LBM_F64: return launch_step_f64(h->d.Q, h->d.mode, kind, h->variant, p, h->st);
        case LBM_F32: return launch_step_f32(h->d.Q, h->d.mode, kind, h->variant, p, h->st);
        case LBM_F16: return launch_step_f16(h->d.Q, h->d.mode, kind, h->variant, p, h->st);
        default: return launch_step_bf16(h->d.Q, h->d.mode, kind, h->variant, p, h->st);
    }
}

// buf[0] holds f^N at each point's own index: collide it into buf[1].
int start_state(lbm_handle* h, bool reset) {
    if (reset) {
        CK(h, cudaMemsetAsync(h->nw_acc, 0, sizeof(double) * 3 * (h->g.nnw + 1), h->st));
        CK(h, cudaMemsetAsync(h->nw_accm, 0, sizeof(double) * (h->g.nnw + 1), h->st));
        CK(h, cudaMemsetAsync(h->nw_wss, 0, sizeof(double) * (h->g.nnw + 1), h->st));
        CK(h, cudaMemsetAsync(h->nw_accf, 0, sizeof(float2) * 4 * (h->g.nnw + 1), h->st));
        CK(h, cudaMemsetAsync(h->nw_wssf, 0, sizeof(float) * (h->g.nnw + 1), h->st));
        CK(h, cudaMemsetAsync(h->nw_ring, 0, sizeof(float) * kRingSlots * 4 * (h->g.nnw + 1), h->st));
        h->wss_from_ckpt = false;
        h->steps = 0;
    }
    int64_t sl[2] = {h->steps, h->steps};
    CK(h, cudaMemcpyAsync(h->slots, sl, sizeof(sl), cudaMemcpyHostToDevice, h->st));
    CK(h, cudaMemsetAsync(h->flags, 0, sizeof(unsigned), h->st));
    if (h->bar) CK(h, cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), h->st));
    StepParams p = make_params(h, 1);
    CK(h, launch(h, 1, p));
    h->cur = 1;
    h->since_start = 0;
    drop_graph(h);  // the graph's buffer roles depend on cur
    CK(h, cudaStreamSynchronize(h->st));
    h->has_state = true;
    return LBM_OK;
}

static_assert(LBM_FLAG_NONFINITE == FLAG_NONFINITE && LBM_FLAG_BOUNDS == FLAG_BOUNDS, "flag values");
static_assert(LBM_NUM_VARIANTS == kNumVariants, "variant count");

int check_flags(lbm_handle* h) {
    unsigned f = 0;
    CK(h, cudaMemcpyAsync(&f, h->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (f & FLAG_TIMEOUT) {
        // a bounded wait gave up; clear the flag and a barrier left half-arrived
        CK(h, cudaMemsetAsync(h->flags, 0, sizeof(unsigned), h->st));
        if (h->bar) CK(h, cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), h->st));
        CK(h, cudaStreamSynchronize(h->st));
        return fail(h, LBM_ERR_CUDA,
                    "a step kernel's bounded wait gave up (a tiled step's bulk copy or a persistent launch's grid "
                    "barrier)");
    }
    if (f & FLAG_BOUNDS) {
        CK(h, cudaMemsetAsync(h->flags, 0, sizeof(unsigned), h->st));
        CK(h, cudaStreamSynchronize(h->st));
        return fail(h, LBM_ERR_CUDA,
                    "a step kernel's index fell outside its array (bounds-checked build; the access was skipped)");
    }
    if (f & FLAG_NONFINITE)
        return fail(h, LBM_ERR_NONFINITE, "a density became NaN/Inf: the run diverged (check tau and the inlet)");
    return LBM_OK;
}

int one_step(lbm_handle* h) {
    StepParams p = make_params(h, 0);
    CK(h, launch(h, 0, p));
    h->cur = 1 - h->cur;
    h->steps++;
    h->since_start++;
    return LBM_OK;
}

// A persistent launch of n (even) steps from the current state (n = 0:
// only the kernel's occupancy query); cur and the counter parity are left
// as they were.
cudaError_t multi_launch(lbm_handle* h, int n) {
    const StepParams even = make_params(h, 0);
    h->cur = 1 - h->cur;
    h->steps++;
    const StepParams odd = make_params(h, 0);
    h->cur = 1 - h->cur;
    h->steps--;
    switch (h->d.precision) {
        case LBM_F64: return launch_multi_f64(h->d.Q, h->d.mode, even, odd, n, h->bar, h->st);
        case LBM_F32: return launch_multi_f32(h->d.Q, h->d.mode, even, odd, n, h->bar, h->st);
        case LBM_F16: return launch_multi_f16(h->d.Q, h->d.mode, even, odd, n, h->bar, h->st);
        default: return launch_multi_bf16(h->d.Q, h->d.mode, even, odd, n, h->bar, h->st);
    }
}

// One persistent launch of h->persist steps.
int multi_steps(lbm_handle* h) {
    const int n = h->persist;
    const cudaError_t e = multi_launch(h, n);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("persistent step launch: ") + cudaGetErrorString(e));
    h->launches++;
    h->steps += n;
    h->since_start += n;
    return LBM_OK;
}

bool persist_ok(const lbm_handle* h) { return (int64_t)h->d.Q * h->stride < ((int64_t)1 << 31); }

// Capture graph_steps (even) launches starting at the current parity.
int build_graph(lbm_handle* h) {
    drop_graph(h);
    const int64_t steps0 = h->steps, since0 = h->since_start, launches0 = h->launches;
    const int cur0 = h->cur;
    cudaGraph_t graph = nullptr;
    // the persistent kernel's occupancy query runs here, outside the capture
    // (an error resurfaces at the captured launch)
    if (h->persist > 0 && multi_launch(h, 0) != cudaSuccess) (void)cudaGetLastError();
    CK(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < h->graph_steps;) {
        if (h->persist > 0) {
            // graph_steps is a multiple of persist (lbm_set_persistent / lbm_set_graph_steps)
            int rc = multi_steps(h);
            if (rc) {
                cudaStreamEndCapture(h->st, &graph);
                if (graph) cudaGraphDestroy(graph);
                h->steps = steps0;
                h->since_start = since0;
                h->launches = launches0;
                return rc;
            }
            k += h->persist;
            continue;
        }
        StepParams p = make_params(h, 0);
        cudaError_t e = launch(h, 0, p);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(h->st, &graph);
            if (graph) cudaGraphDestroy(graph);
            h->steps = steps0;
            h->cur = cur0;
            h->launches = launches0;
            return fail(h, LBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        h->cur = 1 - h->cur;
        h->steps++;
        ++k;
    }
    CK(h, cudaStreamEndCapture(h->st, &graph));
    cudaError_t e = cudaGraphInstantiate(&h->gexec, graph, 0);
    cudaGraphDestroy(graph);
    h->steps = steps0;
    h->since_start = since0;
    h->cur = cur0;
    h->launches = launches0;
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    h->gexec_parity = (int)(steps0 & 1);
    h->gexec_cur = cur0;
    return LBM_OK;
}

// Read-out launch: post-boundary f (optional FP64 copy) + per-block sums.
int readout(lbm_handle* h, bool want_f) {
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state: call lbm_init_equilibrium / lbm_set_geometry first");
    if (want_f && !h->out_f) CK(h, dalloc(h, &h->out_f, sizeof(double) * h->g.nact * h->d.Q));
    StepParams p = make_params(h, 2);
    p.out_f = want_f ? h->out_f : nullptr;
    CK(h, launch(h, 2, p));
    CK(h, reduce_partials(h->partials, h->nblocks, h->sums, h->st));
    return LBM_OK;
}

bool read_stl(const char* path, std::vector<double>& out) {
    std::FILE* fp = std::fopen(path, "r");
    if (!fp) return false;
    std::vector<std::string> lines;
    {
        std::string cur;
        char buf[4096];
        while (std::fgets(buf, sizeof(buf), fp)) {
            cur += buf;
            if (!cur.empty() && cur.back() == '\n') {
                cur.pop_back();
                lines.push_back(cur);
                cur.clear();
            }
        }
        if (!cur.empty()) lines.push_back(cur);
    }
    std::fclose(fp);
    auto tok = [](const std::string& s) {
        std::vector<std::string> t;
        size_t i = 0;
        while (i < s.size()) {
            while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) ++i;
            size_t j = i;
            while (j < s.size() && s[j] != ' ' && s[j] != '\t' && s[j] != '\r') ++j;
            if (j > i) t.push_back(s.substr(i, j - i));
            i = j;
        }
        return t;
    };
    auto num = [](const std::string& s, double& v) {
        char* end = nullptr;
        v = std::strtod(s.c_str(), &end);
        return end && *end == '\0' && end != s.c_str();
    };
    // facet normal / outer loop / 3 vertex / endloop / endfacet, in order
    // (GeometryReader.cpp:50-110); a malformed facet is skipped
    size_t i = 0, n = lines.size();
    while (i < n) {
        auto t = tok(lines[i++]);
        double nn[3];
        if (t.size() < 5 || t[0] != "facet" || t[1] != "normal" || !num(t[2], nn[0]) || !num(t[3], nn[1]) ||
            !num(t[4], nn[2]))
            continue;
        if (i >= n) break;
        t = tok(lines[i++]);
        if (t.size() < 2 || t[0] != "outer" || t[1] != "loop") continue;
        double v[9];
        int got = 0;
        for (int k = 0; k < 3 && i < n; ++k) {
            t = tok(lines[i++]);
            if (t.size() < 4 || t[0] != "vertex" || !num(t[1], v[3 * k]) || !num(t[2], v[3 * k + 1]) ||
                !num(t[3], v[3 * k + 2]))
                break;
            ++got;
        }
        if (got < 3 || i >= n) continue;
        t = tok(lines[i++]);
        if (t.empty() || t[0] != "endloop" || i >= n) continue;
        t = tok(lines[i++]);
        if (t.empty() || t[0] != "endfacet") continue;
        out.insert(out.end(), v, v + 9);
        out.insert(out.end(), nn, nn + 3);
    }
    return true;
}

void reference_bbox(const double* t, int64_t ntri, double spacing, double* bb, int* dims) {
    double mnx = INFINITY, mny = INFINITY, mnz = INFINITY, mxx = -INFINITY, mxy = -INFINITY, mxz = -INFINITY;
    for (int64_t k = 0; k < ntri; ++k) {
        const double* r = t + 12 * k;
        // the y and z extremes ignore the third vertex (ComplexGeometry.cpp:147-151)
        mnx = std::min(std::min(std::min(mnx, r[0]), r[3]), r[6]);
        mny = std::min(std::min(mny, r[1]), r[4]);
        mnz = std::min(std::min(mnz, r[2]), r[5]);
        mxx = std::max(std::max(std::max(mxx, r[0]), r[3]), r[6]);
        mxy = std::max(std::max(mxy, r[1]), r[4]);
        mxz = std::max(std::max(mxz, r[2]), r[5]);
    }
    bb[0] = mnx; bb[1] = mxx; bb[2] = mny; bb[3] = mxy; bb[4] = mnz; bb[5] = mxz;
    dims[0] = (int)std::ceil((mxx - mnx) / spacing) + 1;
    dims[1] = (int)std::ceil((mxy - mny) / spacing) + 1;
    dims[2] = (int)std::ceil((mxz - mnz) / spacing);
}

// Pull segments.  With populations stored by active index a, the source of
// population q at node a is the active index of point x_a - c_q.  Along an
// x-run that index is a + delta_q with delta_q constant; a segment is a
// maximal stretch of consecutive active nodes whose valid (non-missing)
// offsets agree for every q.  Output: per active node its segment, per
// segment Q offsets (0 where no node of the segment has that source), each
// row padded with zeros to kDeltaRow<Q> entries so that the step kernel
// reads it with 16-byte loads.
template <int Q>
void build_segments_q(const uint8_t* mask, int nx, int ny, int nz, int64_t& nact, std::vector<int32_t>& seg_of,
                      std::vector<int32_t>& delta) {
    const int64_t nxy = (int64_t)nx * ny, npts = nxy * nz;
    std::vector<int32_t> aidx((size_t)npts);
    int64_t a = 0;
    for (int64_t n = 0; n < npts; ++n) aidx[n] = mask[n] ? (int32_t)a++ : -1;
    nact = a;
    seg_of.assign((size_t)nact, 0);
    delta.clear();
    int32_t cur[Q];
    bool has[Q];
    int64_t seg = -1;
    auto flush = [&]() {
        for (int q = 0; q < Q; ++q) delta.push_back(has[q] ? cur[q] : 0);
        for (int q = Q; q < kDeltaRow<Q>; ++q) delta.push_back(0);
    };
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t n = (int64_t)k * nxy + (int64_t)j * nx + i;
                if (!mask[n]) continue;
                const int32_t an = aidx[n];
                int32_t d[Q];
                bool v[Q];
                bool fresh = seg < 0;
                for (int q = 0; q < Q; ++q) {
                    const int x = i - Lat<Q>::cx(q), y = j - Lat<Q>::cy(q), z = k - Lat<Q>::cz(q);
                    v[q] = x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz &&
                           mask[(int64_t)z * nxy + (int64_t)y * nx + x];
                    d[q] = v[q] ? aidx[(int64_t)z * nxy + (int64_t)y * nx + x] - an : 0;
                    if (!fresh && v[q] && has[q] && d[q] != cur[q]) fresh = true;
                }
                if (fresh) {
                    if (seg >= 0) flush();
                    ++seg;
                    for (int q = 0; q < Q; ++q) has[q] = false;
                }
                for (int q = 0; q < Q; ++q)
                    if (v[q] && !has[q]) { cur[q] = d[q]; has[q] = true; }
                seg_of[an] = (int32_t)seg;
            }
    if (seg >= 0) flush();
}

void build_segments(int Q, const uint8_t* mask, int nx, int ny, int nz, int64_t& nact, std::vector<int32_t>& seg_of,
                    std::vector<int32_t>& delta) {
    if (Q == 19) build_segments_q<19>(mask, nx, ny, nz, nact, seg_of, delta);
    else build_segments_q<27>(mask, nx, ny, nz, nact, seg_of, delta);
}

// FP32 copy of the normals [3][nn] with plane stride `stride`.
std::vector<float> float_normals(const std::vector<double>& nd, int64_t nn, int64_t stride) {
    std::vector<float> nf(3 * stride, 0.f);
    for (int a = 0; a < 3; ++a)
        for (int64_t k = 0; k < nn; ++k) nf[a * stride + k] = (float)nd[a * nn + k];
    return nf;
}

// Plan of the tiled step kernel: per tile of kTileNodes active nodes and
// population plane q, the window of plane q holding every valid pull source
// of the tile's nodes (widened to 16-byte boundaries); the tile's pull
// segments and next-to-wall entries; the shared-memory layout of a pipeline
// stage.  Returns false (no plan) when a stage does not fit.
template <int Q>
bool build_tile_plan_q(const uint8_t* mask, int nx, int ny, int nz, int64_t nact, int64_t stride, int es,
                       const std::vector<int32_t>& seg_of, const std::vector<int32_t>& delta,
                       const std::vector<int32_t>& sp_of_act, int64_t nnw, std::vector<int32_t>& plan, TileGeom& G) {
    constexpr int T = kTileNodes, DR = kDeltaRow<Q>, PI = 2 * Q + kTilePlanExtra;
    const int A = 16 / es;  // elements per 16 bytes
    const int64_t ntiles = ceil_div(nact, T);
    const int64_t nxy = (int64_t)nx * ny;
    std::vector<int64_t> lo((size_t)ntiles * Q, INT64_MAX), hi((size_t)ntiles * Q, -1);
    int64_t an = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                if (!mask[(int64_t)k * nxy + (int64_t)j * nx + i]) continue;
                const int32_t* d = delta.data() + (int64_t)seg_of[an] * DR;
                const int64_t t = an / T;
                for (int q = 0; q < Q; ++q) {
                    const int x = i - Lat<Q>::cx(q), y = j - Lat<Q>::cy(q), z = k - Lat<Q>::cz(q);
                    if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz ||
                        !mask[(int64_t)z * nxy + (int64_t)y * nx + x])
                        continue;
                    const int64_t src = an + d[q];
                    int64_t& l = lo[t * Q + q];
                    int64_t& h = hi[t * Q + q];
                    if (src < l) l = src;
                    if (src > h) h = src;
                }
                ++an;
            }
    plan.assign((size_t)ntiles * PI, 0);
    int64_t wcap = A, segmax = 1, nwcap = 4;
    for (int64_t t = 0; t < ntiles; ++t) {
        int32_t* pl = plan.data() + t * PI;
        for (int q = 0; q < Q; ++q) {
            const int64_t h = hi[t * Q + q];
            if (h < 0) continue;
            const int64_t l0 = lo[t * Q + q] / A * A, h1 = ceil_div(h + 1, A) * A;
            if (h1 > stride) return false;
            pl[q] = (int32_t)l0;
            pl[Q + q] = (int32_t)(h1 - l0);
            wcap = std::max(wcap, h1 - l0);
        }
        const int64_t a0 = t * T, a1 = std::min(nact, a0 + T) - 1;
        pl[2 * Q] = seg_of[a0];
        pl[2 * Q + 1] = seg_of[a1] - seg_of[a0] + 1;
        segmax = std::max<int64_t>(segmax, pl[2 * Q + 1]);
        int64_t smin = INT64_MAX, smax = -1;
        for (int64_t a = a0; a <= a1; ++a)
            if (sp_of_act[a] >= 0 && sp_of_act[a] < nnw) {
                smin = std::min<int64_t>(smin, sp_of_act[a]);
                smax = std::max<int64_t>(smax, sp_of_act[a]);
            }
        if (smax >= 0) {
            pl[2 * Q + 2] = (int32_t)(smin / 4 * 4);
            pl[2 * Q + 3] = (int32_t)(ceil_div(smax + 1, 4) * 4 - smin / 4 * 4);
            nwcap = std::max<int64_t>(nwcap, pl[2 * Q + 3]);
        }
    }
    const int segcap = (int)std::min<int64_t>(segmax, 64);
    for (int64_t t = 0; t < ntiles; ++t) {
        int32_t* pl = plan.data() + t * PI;
        pl[2 * Q + 1] = std::min(pl[2 * Q + 1], segcap);  // the rest read their rows from global memory
    }
    wcap = ceil_div(wcap, 8) * 8;
    auto al = [](int64_t v) { return (int)ceil_div(v, 128) * 128; };
    TileGeom g{};
    g.ntiles = ntiles;
    g.wcap = (int)wcap;
    g.segcap = segcap;
    g.nwcap = (int)nwcap;
    g.off_pull = 0;
    g.off_own = al(g.off_pull + (int64_t)Q * wcap * es);
    g.off_word = al(g.off_own + (int64_t)Q * T * es);
    g.off_sp = al(g.off_word + (int64_t)T * 8);
    g.off_delta = al(g.off_sp + (int64_t)T * 4);
    g.off_nrm = al(g.off_delta + (int64_t)segcap * DR * 4);
    g.off_hdr = al(g.off_nrm + 3 * nwcap * 4);
    g.stage_bytes = al(g.off_hdr + (Q + 3) * 4);
    // deepest pipeline and most CTAs per SM that fit 227 KB per CTA / 228 KB per SM
    const int choices[4][2] = {{3, 2}, {2, 2}, {3, 1}, {2, 1}};
    for (const auto& c : choices) {
        const int smem = c[0] * g.stage_bytes + c[0] * 8;
        if (smem <= 232448 && c[1] * (smem + 1024) <= 233472) {
            g.nstage = c[0];
            g.ctas_per_sm = c[1];
            g.smem_bytes = smem;
            G = g;
            return true;
        }
    }
    return false;
}

const uint32_t kCkptMagic = 0x4c424d43;  // "CMBL"
const uint32_t kCkptVersion = 3;  // 2: boundary list next-to-wall first; 3: every inlet waveform

}  // namespace

void lbm::set_last_global_error(const char* msg) { g_err = msg ? msg : ""; }

// ===========================================================================

extern "C" {

const char* lbm_last_global_error(void) { return g_err.c_str(); }

const char* lbm_last_error(const lbm_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

lbm_status lbm_read_stl_ascii(const char* path, double* tri12, int64_t* ntri) {
    if (!path || !ntri) return fail(nullptr, LBM_ERR_ARG, "null path or count");
    std::vector<double> v;
    if (!read_stl(path, v)) return fail(nullptr, LBM_ERR_IO, std::string("cannot open ") + path);
    const int64_t n = (int64_t)(v.size() / 12);
    if (tri12) {
        const int64_t m = std::min(n, *ntri);
        std::memcpy(tri12, v.data(), sizeof(double) * 12 * m);
    }
    *ntri = n;
    return LBM_OK;
}

lbm_status lbm_voxelize(const double* tri12, int64_t ntri, lbm_vox_desc* desc, uint8_t* mask_out) {
    if (!desc || (ntri > 0 && !tri12) || ntri < 0) return fail(nullptr, LBM_ERR_ARG, "null descriptor or triangles");
    if (!(desc->spacing > 0)) return fail(nullptr, LBM_ERR_ARG, "spacing must be > 0");
    if (desc->reference_bbox) {
        if (ntri == 0) return fail(nullptr, LBM_ERR_ARG, "the reference bbox needs at least one triangle");
        reference_bbox(tri12, ntri, desc->spacing, desc->bbox, desc->dims);
        desc->origin[0] = desc->bbox[0];
        desc->origin[1] = desc->bbox[2];
        desc->origin[2] = desc->bbox[4];
    }
    const int nx = desc->dims[0], ny = desc->dims[1], nz = desc->dims[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return fail(nullptr, LBM_ERR_ARG, "empty lattice");
    if (!mask_out) return LBM_OK;
    const int64_t npts = (int64_t)nx * ny * nz;
    cudaStream_t st = nullptr;
    double* d_tri = nullptr;
    uint8_t* d_mask = nullptr;
    std::string err;
    auto cleanup = [&]() {
        if (d_tri) cudaFree(d_tri);
        if (d_mask) cudaFree(d_mask);
        if (st) cudaStreamDestroy(st);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d_tri, sizeof(double) * 12 * (ntri > 0 ? ntri : 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_mask, npts);
    if (e == cudaSuccess && ntri > 0)
        e = cudaMemcpyAsync(d_tri, tri12, sizeof(double) * 12 * ntri, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_mask, 0, npts, st);
    VoxResult res{};
    if (e == cudaSuccess) {
        e = voxelize_device(d_tri, ntri, desc->bbox, desc->origin, desc->spacing, desc->dims, d_mask, &res, st, &err);
    } else {
        err = cudaGetErrorString(e);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(mask_out, d_mask, npts, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess)
        return fail(nullptr, e == cudaErrorMemoryAllocation ? LBM_ERR_ALLOC : LBM_ERR_CUDA,
                    "voxelize: " + (err.empty() ? std::string(cudaGetErrorString(e)) : err));
    desc->fluid_count = res.fluid;
    desc->ray_tests = res.tests;
    return LBM_OK;
}

lbm_status lbm_create(const lbm_desc* desc, lbm_handle** out) {
    if (!desc || !out) return fail(nullptr, LBM_ERR_ARG, "null descriptor or output");
    if (desc->Q != 19 && desc->Q != 27) return fail(nullptr, LBM_ERR_ARG, "Q must be 19 or 27");
    if (elem_size(desc->precision) == 0) return fail(nullptr, LBM_ERR_ARG, "unknown precision");
    if (desc->mode != LBM_PARITY && desc->mode != LBM_PHYSICS) return fail(nullptr, LBM_ERR_ARG, "unknown mode");
    if (!(desc->tau > 0.5)) return fail(nullptr, LBM_ERR_ARG, "tau must be > 0.5 (BGK stability)");
    if (desc->collision != LBM_COLLISION_BGK && desc->collision != LBM_COLLISION_REGULARIZED)
        return fail(nullptr, LBM_ERR_ARG, "collision must be LBM_COLLISION_BGK or LBM_COLLISION_REGULARIZED");
    if (!(desc->spacing > 0)) return fail(nullptr, LBM_ERR_ARG, "spacing must be > 0");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, LBM_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (desc->device < 0 || desc->device >= ndev) return fail(nullptr, LBM_ERR_ARG, "device ordinal out of range");
    lbm_handle* h = new lbm_handle();
    h->d = *desc;
    if (h->d.tawss_div == 0.0) h->d.tawss_div = 0.9;
    // FP64 keeps every population in two registers: start it on the
    // unconstrained shape, the FP32-arithmetic formats on the 40-register one
    h->variant = h->d.precision == LBM_F64 ? 4 : 0;
    e = cudaSetDevice(desc->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->slots, 2 * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->flags, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&h->wave_off, sizeof(int64_t) * LBM_MAX_WAVES);
    if (e == cudaSuccess) e = cudaMalloc(&h->wave_len, sizeof(int64_t) * LBM_MAX_WAVES);
    if (e != cudaSuccess) {
        int rc = fail(nullptr, LBM_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
        lbm_destroy(h);
        return rc;
    }
    h->waves.assign(1, std::vector<double>(1, 0.0));
    if (upload_waves(h) != LBM_OK) {
        lbm_destroy(h);
        return LBM_ERR_CUDA;
    }
    *out = h;
    return LBM_OK;
}

lbm_status lbm_destroy(lbm_handle* h) {
    if (!h) return LBM_OK;
    cudaSetDevice(h->d.device);
    if (h->st) cudaStreamSynchronize(h->st);
    free_geometry(h);
    if (h->slots) cudaFree(h->slots);
    if (h->flags) cudaFree(h->flags);
    if (h->bar) cudaFree(h->bar);
    if (h->amp) cudaFree(h->amp);
    if (h->wave_off) cudaFree(h->wave_off);
    if (h->wave_len) cudaFree(h->wave_len);
    if (h->cst) cudaStreamSynchronize(h->cst);
    if (h->amp_pinned) cudaFreeHost(h->amp_pinned);
    for (cudaEvent_t e : {h->ev_ready, h->ev_copied[0], h->ev_copied[1], h->ev_table})
        if (e) cudaEventDestroy(e);
    if (h->cst) cudaStreamDestroy(h->cst);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return LBM_OK;
}

lbm_status lbm_set_geometry(lbm_handle* h, const uint8_t* mask, const int dims[3], const lbm_bc_spec* bc, int nbc) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, mask && dims, LBM_ERR_ARG, "null mask or dims");
    REQUIRE(h, dims[0] > 0 && dims[1] > 0 && dims[2] > 0, LBM_ERR_ARG, "empty lattice");
    REQUIRE(h, nbc >= 0 && nbc <= LBM_MAX_BC && (nbc == 0 || bc), LBM_ERR_ARG, "0..256 boundary conditions");
    const int64_t npts = (int64_t)dims[0] * dims[1] * dims[2];
    REQUIRE(h, npts < (int64_t)1 << 31, LBM_ERR_ARG, "lattice too large (more than 2^31 points)");
    for (int b = 0; b < nbc; ++b) {
        REQUIRE(h, bc[b].kind >= LBM_BC_REF_INLET && bc[b].kind <= LBM_BC_PRESSURE, LBM_ERR_ARG, "unknown bc kind");
        REQUIRE(h, bc[b].face >= 0 && bc[b].face <= 5, LBM_ERR_ARG, "face must be 0..5");
        REQUIRE(h, bc[b].kind != LBM_BC_PRESSURE || bc[b].value > 0, LBM_ERR_ARG, "pressure bc needs density > 0");
        REQUIRE(h, bc[b].profile == 0 || bc[b].R > 0, LBM_ERR_ARG, "profile radius must be > 0");
        REQUIRE(h, bc[b].wave >= 0 && bc[b].wave < LBM_MAX_WAVES, LBM_ERR_ARG, "waveform index out of range");
    }
    CK(h, cudaSetDevice(h->d.device));
    CK(h, cudaStreamSynchronize(h->st));
    free_geometry(h);
    h->nx = dims[0]; h->ny = dims[1]; h->nz = dims[2];
    h->npts = npts;
    int64_t nact = 0;
    std::vector<int32_t> seg_of, delta;
    build_segments(h->d.Q, mask, h->nx, h->ny, h->nz, nact, seg_of, delta);
    REQUIRE(h, nact < (int64_t)1 << 31, LBM_ERR_ARG, "too many active nodes");
    h->nseg = (int64_t)delta.size() / (h->d.Q == 19 ? kDeltaRow<19> : kDeltaRow<27>);
    h->stride = ceil_div(nact > 0 ? nact : 1, 128) * 128;
    CK(h, dalloc(h, &h->seg_delta, sizeof(int32_t) * (delta.size() + 1)));
    if (!delta.empty())
        CK(h, cudaMemcpyAsync(h->seg_delta, delta.data(), sizeof(int32_t) * delta.size(), cudaMemcpyHostToDevice, h->st));
    uint8_t* d_mask = nullptr;
    int32_t* d_seg = nullptr;
    CK(h, cudaMalloc(&d_mask, npts));
    cudaError_t e = cudaMalloc(&d_seg, sizeof(int32_t) * (nact + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_mask, mask, npts, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess && nact)
        e = cudaMemcpyAsync(d_seg, seg_of.data(), sizeof(int32_t) * nact, cudaMemcpyHostToDevice, h->st);
    std::string err;
    if (e == cudaSuccess)
        e = build_geometry(h->d.Q, d_mask, h->nx, h->ny, h->nz, bc, nbc, h->d.origin, h->d.spacing, d_seg, h->g,
                           h->st, err);
    cudaFree(d_mask);
    if (d_seg) cudaFree(d_seg);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, "set_geometry: " + (err.empty() ? cudaGetErrorString(e) : err));
    REQUIRE(h, h->g.nact < (int64_t)1 << 31, LBM_ERR_ARG, "too many active nodes");
    h->nbc = nbc;
    h->bc.assign(nbc, BCDev{});
    for (int b = 0; b < nbc; ++b) {
        h->bc[b].kind = bc[b].kind;
        h->bc[b].face = bc[b].face;
        h->bc[b].value = bc[b].value;
        h->bc[b].profile = bc[b].profile;
        h->bc[b].c1 = bc[b].c1;
        h->bc[b].c2 = bc[b].c2;
        h->bc[b].R = bc[b].R;
        h->bc[b].wave = bc[b].wave;
        h->bc[b].value_m1 = (float)(bc[b].value - 1.0);
    }
    CK(h, dalloc(h, &h->bct, sizeof(BCDev) * (nbc + 1)));
    if (nbc) CK(h, cudaMemcpyAsync(h->bct, h->bc.data(), sizeof(BCDev) * nbc, cudaMemcpyHostToDevice, h->st));
    CK(h, dalloc(h, &h->sp_flux, sizeof(double) * (h->g.nsp + 1)));
    const int Q = h->d.Q;
    const size_t es = elem_size(h->d.precision), rs = real_size(h->d.precision);
    CK(h, dalloc(h, &h->buf[0], es * Q * h->stride));
    CK(h, dalloc(h, &h->buf[1], es * Q * h->stride));
    CK(h, cudaMemsetAsync(h->buf[0], 0, es * Q * h->stride, h->st));
    CK(h, cudaMemsetAsync(h->buf[1], 0, es * Q * h->stride, h->st));
    if (h->d.mode == LBM_PARITY) {
        CK(h, dalloc(h, &h->stale, rs * Q * (h->g.nsp + 1)));
        CK(h, dalloc(h, &h->nw_prev, rs * 4 * (h->g.nnw + 1)));
    }
    CK(h, dalloc(h, &h->nw_n, sizeof(double) * 3 * (h->g.nnw + 1)));
    CK(h, cudaMemsetAsync(h->nw_n, 0, sizeof(double) * 3 * (h->g.nnw + 1), h->st));
    CK(h, dalloc(h, &h->nw_wss, sizeof(double) * (h->g.nnw + 1)));
    CK(h, dalloc(h, &h->nw_acc, sizeof(double) * 3 * (h->g.nnw + 1)));
    CK(h, dalloc(h, &h->nw_accm, sizeof(double) * (h->g.nnw + 1)));
    h->nw_stride = ceil_div(h->g.nnw + 1, 4) * 4;  // 16-byte planes: the tiled kernel copies them in bulk
    CK(h, dalloc(h, &h->nw_nf, sizeof(float) * 3 * h->nw_stride));
    CK(h, cudaMemsetAsync(h->nw_nf, 0, sizeof(float) * 3 * h->nw_stride, h->st));
    CK(h, dalloc(h, &h->nw_wssf, sizeof(float) * (h->g.nnw + 1)));
    CK(h, dalloc(h, &h->nw_accf, sizeof(float2) * 4 * (h->g.nnw + 1)));
    CK(h, dalloc(h, &h->nw_ring, sizeof(float) * kRingSlots * 4 * (h->g.nnw + 1)));
    if (h->d.mode == LBM_PHYSICS && h->d.precision != LBM_F64 && (int64_t)Q * h->stride < ((int64_t)1 << 31)) {
        // compact step kernel: absolute pull rows and per-warp blocks
        const int64_t rows = h->nseg * (Q == 19 ? kDeltaRow<19> : kDeltaRow<27>);
        CK(h, dalloc(h, &h->warp_block, sizeof(uint32_t) * kWarpBlockWords * block_warps(h->g.nact)));
        CK(h, dalloc(h, &h->seg_abs, sizeof(int32_t) * (rows + 4)));
        CK(h, build_compact_meta(Q, h->g.act_word, h->g.sp_of_act, h->g.nact, h->g.nnw, h->seg_delta, h->nseg,
                                 h->stride, h->warp_block, h->seg_abs, h->st));
    }
    h->nblocks = ceil_div(h->g.nact, kStepThreads);
    CK(h, dalloc(h, &h->partials, sizeof(double) * kPartialStride * (h->nblocks + 1)));
    CK(h, dalloc(h, &h->sums, sizeof(double) * kPartialStride));
    h->geo_bytes += h->npts * 5 + h->g.nsp * 25 + h->g.nact * 28;  // lists from setup
    h->has_geo = true;
    // counts
    std::vector<uint8_t> spc(h->g.nsp);
    h->sp_bc.assign(h->g.nsp, -1);
    if (h->g.nsp) {
        CK(h, cudaMemcpyAsync(spc.data(), h->g.sp_cls, h->g.nsp, cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaMemcpyAsync(h->sp_bc.data(), h->g.sp_bc, sizeof(int32_t) * h->g.nsp, cudaMemcpyDeviceToHost,
                              h->st));
    }
    CK(h, cudaStreamSynchronize(h->st));
    lbm_counts c{};
    c.points = h->npts;
    c.active = h->g.nact;
    c.next_to_wall = h->g.nnw;
    c.special = h->g.nsp;
    c.segments = h->nseg;
    int64_t bnd = 0;
    for (int64_t e = 0; e < h->g.nsp; ++e) {
        const uint8_t v = spc[e];
        if (v == CLS_WALL) c.wall++;
        else if (v >= CLS_BC0 && h->sp_bc[e] >= 0 && h->sp_bc[e] < LBM_MAX_BC) c.bc[h->sp_bc[e]]++;
        if (v >= CLS_WALL) bnd++;
    }
    c.fluid = h->g.nact - bnd;
    h->counts = c;
    // plan of the tiled step kernel (physics mode, FP32-arithmetic formats)
    if (h->d.mode == LBM_PHYSICS && h->d.precision != LBM_F64 && h->g.nact > 0) {
        std::vector<int32_t> spa(h->g.nact);
        CK(h, cudaMemcpyAsync(spa.data(), h->g.sp_of_act, sizeof(int32_t) * h->g.nact, cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaStreamSynchronize(h->st));
        std::vector<int32_t> plan;
        TileGeom G{};
        const int es = (int)elem_size(h->d.precision);
        const bool ok = Q == 19 ? build_tile_plan_q<19>(mask, h->nx, h->ny, h->nz, h->g.nact, h->stride, es, seg_of,
                                                         delta, spa, h->g.nnw, plan, G)
                                : build_tile_plan_q<27>(mask, h->nx, h->ny, h->nz, h->g.nact, h->stride, es, seg_of,
                                                         delta, spa, h->g.nnw, plan, G);
        if (ok) {
            CK(h, dalloc(h, &h->tile_plan, sizeof(int32_t) * plan.size()));
            CK(h, cudaMemcpyAsync(h->tile_plan, plan.data(), sizeof(int32_t) * plan.size(), cudaMemcpyHostToDevice,
                                  h->st));
            CK(h, cudaStreamSynchronize(h->st));
            h->tile = G;
        }
    }
    return lbm_init_equilibrium(h);
}

lbm_status lbm_set_normals_from_surface(lbm_handle* h, const double* tri12, int64_t ntri) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, ntri >= 0 && (ntri == 0 || tri12), LBM_ERR_ARG, "null triangles");
    CK(h, cudaSetDevice(h->d.device));
    double* d_tri = nullptr;
    CK(h, cudaMalloc(&d_tri, sizeof(double) * 12 * (ntri > 0 ? ntri : 1)));
    cudaError_t e = cudaSuccess;
    if (ntri > 0) e = cudaMemcpyAsync(d_tri, tri12, sizeof(double) * 12 * ntri, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = surface_normals(d_tri, ntri, h->g.nw_pt, h->g.nnw, h->nx, h->ny, h->d.origin, h->d.spacing, h->nw_n, h->st);
    if (e == cudaSuccess && h->g.nnw > 0) {
        // FP32 copy for the FP32-arithmetic formats
        std::vector<double> nd(3 * h->g.nnw);
        e = cudaMemcpyAsync(nd.data(), h->nw_n, sizeof(double) * nd.size(), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        const std::vector<float> nf = float_normals(nd, h->g.nnw, h->nw_stride);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->nw_nf, nf.data(), sizeof(float) * nf.size(), cudaMemcpyHostToDevice, h->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(d_tri);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("normals: ") + cudaGetErrorString(e));
    return LBM_OK;
}

lbm_status lbm_set_normals_from_surface_box(lbm_handle* h, const double* tri12, int64_t ntri, const double lo[3],
                                            const double hi[3]) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, ntri >= 0 && (ntri == 0 || tri12) && lo && hi, LBM_ERR_ARG, "null triangles or box");
    CK(h, cudaSetDevice(h->d.device));
    const int64_t nn = h->g.nnw;
    if (nn == 0) return LBM_OK;
    // next-to-wall points inside the box
    std::vector<int64_t> pt(nn), sel_idx, sel_pt;
    CK(h, cudaMemcpyAsync(pt.data(), h->g.nw_pt, sizeof(int64_t) * nn, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    const int64_t nxy = (int64_t)h->nx * h->ny;
    for (int64_t p = 0; p < nn; ++p) {
        const int64_t n = pt[p];
        const int64_t idx[3] = {n % h->nx, (n / h->nx) % h->ny, n / nxy};
        bool in = true;
        for (int a = 0; a < 3; ++a) {
            const double x = h->d.origin[a] + (double)idx[a] * h->d.spacing;
            in = in && lo[a] <= x && x < hi[a];
        }
        if (in) {
            sel_idx.push_back(p);
            sel_pt.push_back(n);
        }
    }
    const int64_t m = (int64_t)sel_pt.size();
    if (m == 0) return LBM_OK;
    double* d_tri = nullptr;
    int64_t* d_pt = nullptr;
    double* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_tri, sizeof(double) * 12 * (ntri > 0 ? ntri : 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_pt, sizeof(int64_t) * m);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(double) * 3 * m);
    if (e == cudaSuccess && ntri > 0)
        e = cudaMemcpyAsync(d_tri, tri12, sizeof(double) * 12 * ntri, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_pt, sel_pt.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = surface_normals(d_tri, ntri, d_pt, m, h->nx, h->ny, h->d.origin, h->d.spacing, d_out, h->st);
    std::vector<double> part(3 * m), nd(3 * nn);
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_out, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nd.data(), h->nw_n, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    std::vector<float> nf;
    if (e == cudaSuccess) {
        for (int64_t k = 0; k < m; ++k)
            for (int a = 0; a < 3; ++a) nd[a * nn + sel_idx[k]] = part[a * m + k];
        nf = float_normals(nd, nn, h->nw_stride);
        e = cudaMemcpyAsync(h->nw_n, nd.data(), sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, h->st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->nw_nf, nf.data(), sizeof(float) * nf.size(), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(d_tri);
    cudaFree(d_pt);
    cudaFree(d_out);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("normals: ") + cudaGetErrorString(e));
    return LBM_OK;
}

lbm_status lbm_set_wall_distances(lbm_handle* h, const double* tri12, int64_t ntri) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, h->d.mode == LBM_PHYSICS, LBM_ERR_ARG, "interpolated bounce-back is a physics-mode rule");
    REQUIRE(h, ntri >= 0 && (ntri == 0 || tri12), LBM_ERR_ARG, "null triangles");
    CK(h, cudaSetDevice(h->d.device));
    CK(h, cudaStreamSynchronize(h->st));
    drop_graph(h);  // the table pointer is baked into captured launches
    if (ntri == 0) {
        if (h->sp_q) cudaFree(h->sp_q);
        h->sp_q = nullptr;
        return LBM_OK;
    }
    if (!h->sp_q) CK(h, dalloc(h, &h->sp_q, sizeof(float) * h->d.Q * (h->g.nsp + 1)));
    double* d_tri = nullptr;
    CK(h, cudaMalloc(&d_tri, sizeof(double) * 12 * ntri));
    cudaError_t e = cudaMemcpyAsync(d_tri, tri12, sizeof(double) * 12 * ntri, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = wall_distances(h->d.Q, d_tri, ntri, h->g, h->nx, h->ny, h->d.origin, h->d.spacing, h->sp_q, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(d_tri);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("wall distances: ") + cudaGetErrorString(e));
    return LBM_OK;
}

lbm_status lbm_get_wall_distances(lbm_handle* h, int64_t* pt, float* q) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    CK(h, cudaSetDevice(h->d.device));
    const int64_t n = h->g.nsp;
    const int Q = h->d.Q;
    if (pt && n) CK(h, cudaMemcpyAsync(pt, h->g.sp_pt, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, h->st));
    std::vector<float> planes((size_t)Q * n, 0.5f);
    if (q && n && h->sp_q)
        CK(h, cudaMemcpyAsync(planes.data(), h->sp_q, sizeof(float) * Q * n, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (q)
        for (int64_t e = 0; e < n; ++e)
            for (int k = 0; k < Q; ++k) q[e * Q + k] = planes[(size_t)k * n + e];
    return LBM_OK;
}

lbm_status lbm_set_inlet_table(lbm_handle* h, const double* amp, int64_t n) {
    return lbm_set_waveform(h, 0, amp, n);
}

lbm_status lbm_set_waveform(lbm_handle* h, int wave, const double* amp, int64_t n) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, amp && n > 0, LBM_ERR_ARG, "empty amplitude table");
    REQUIRE(h, wave >= 0 && wave < LBM_MAX_WAVES, LBM_ERR_ARG, "waveform index out of range");
    CK(h, cudaSetDevice(h->d.device));
    if ((int)h->waves.size() <= wave) h->waves.resize(wave + 1);
    h->waves[wave].assign(amp, amp + n);
    return upload_waves(h);
}

lbm_status lbm_init_equilibrium(lbm_handle* h) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    CK(h, cudaSetDevice(h->d.device));
    CK(h, init_state(h->d.precision, h->d.Q, 0, h->buf[0], h->stride, nullptr, h->g.nact, h->st));
    return start_state(h, true);
}

lbm_status lbm_set_distributions(lbm_handle* h, const double* f) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, f, LBM_ERR_ARG, "null distributions");
    CK(h, cudaSetDevice(h->d.device));
    const size_t bytes = sizeof(double) * h->g.nact * h->d.Q;
    if (!h->out_f) CK(h, dalloc(h, &h->out_f, bytes));
    CK(h, cudaMemcpyAsync(h->out_f, f, bytes, cudaMemcpyHostToDevice, h->st));
    CK(h, init_state(h->d.precision, h->d.Q, 1, h->buf[0], h->stride, h->out_f, h->g.nact, h->st));
    return start_state(h, false);
}

lbm_status lbm_init_from_macro_device(lbm_handle* h, const float* rho, const float* u, int regularized,
                                      void* stream) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, rho && u, LBM_ERR_ARG, "null rho or u");
    CK(h, cudaSetDevice(h->d.device));
    const int64_t na = h->g.nact;
    if (!h->out_f) CK(h, dalloc(h, &h->out_f, sizeof(double) * na * h->d.Q));
    cudaEvent_t ev = nullptr;
    CK(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->st, ev, 0);
    if (e == cudaSuccess)
        e = warm_start_f(h->d.Q, rho, u, h->g.act_idx, h->g.act_pt, na, h->nx, h->ny, h->nz, h->d.tau, regularized,
                         h->out_f, h->st);
    if (e == cudaSuccess) e = init_state(h->d.precision, h->d.Q, 1, h->buf[0], h->stride, h->out_f, na, h->st);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("init_from_macro_device: ") + cudaGetErrorString(e));
    return start_state(h, true);
}

lbm_status lbm_init_from_macro(lbm_handle* h, const float* rho, const float* u, int regularized) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, rho && u, LBM_ERR_ARG, "null rho or u");
    CK(h, cudaSetDevice(h->d.device));
    const int64_t na = h->g.nact;
    float *d_rho = nullptr, *d_u = nullptr;
    if (!h->out_f) CK(h, dalloc(h, &h->out_f, sizeof(double) * na * h->d.Q));
    CK(h, cudaMalloc(&d_rho, sizeof(float) * (na + 1)));
    cudaError_t e = cudaMalloc(&d_u, sizeof(float) * 3 * (na + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rho, rho, sizeof(float) * na, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_u, u, sizeof(float) * 3 * na, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = warm_start_f(h->d.Q, d_rho, d_u, h->g.act_idx, h->g.act_pt, na, h->nx, h->ny, h->nz, h->d.tau,
                         regularized, h->out_f, h->st);
    if (e == cudaSuccess)
        e = init_state(h->d.precision, h->d.Q, 1, h->buf[0], h->stride, h->out_f, na, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(d_rho);
    if (d_u) cudaFree(d_u);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("init_from_macro: ") + cudaGetErrorString(e));
    return start_state(h, true);
}

lbm_status lbm_step(lbm_handle* h, int nsteps) {
    int rc = lbm_step_async(h, nsteps);
    if (rc) return rc;
    return check_flags(h);
}

lbm_status lbm_check_status(lbm_handle* h) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state: set the geometry first");
    return check_flags(h);
}

lbm_status lbm_step_async(lbm_handle* h, int nsteps) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state: set the geometry first");
    REQUIRE(h, nsteps >= 0, LBM_ERR_ARG, "negative step count");
    CK(h, cudaSetDevice(h->d.device));
    if (nsteps > 0) h->wss_from_ckpt = false;
    REQUIRE(h, h->persist == 0 || persist_ok(h), LBM_ERR_UNSUPPORTED,
            "persistent steps need 32-bit population offsets (Q * stride < 2^31)");
    int left = nsteps;
    // Graph replay: a captured graph bakes the buffer roles (cur) and the
    // counter slot (step parity); both flip every step, so a graph built at
    // one (cur, parity) is valid whenever that pair recurs -- one direct step
    // re-aligns otherwise.
    while (h->graph_steps > 0 && left >= h->graph_steps) {
        if (h->gexec && (h->gexec_parity != (int)(h->steps & 1) || h->gexec_cur != h->cur)) {
            int rc = one_step(h);
            if (rc) return rc;
            --left;
            continue;
        }
        if (!h->gexec) {
            int rc = build_graph(h);
            if (rc) return rc;
        }
        CK(h, cudaGraphLaunch(h->gexec, h->st));
        h->launches += h->persist > 0 ? h->graph_steps / h->persist : h->graph_steps;
        h->steps += h->graph_steps;
        h->since_start += h->graph_steps;
        left -= h->graph_steps;  // even count: cur and parity return to the captured pair
    }
    while (h->persist > 0 && left >= h->persist) {
        int rc = multi_steps(h);
        if (rc) return rc;
        left -= h->persist;
    }
    for (; left > 0; --left) {
        int rc = one_step(h);
        if (rc) return rc;
    }
    return LBM_OK;
}

lbm_status lbm_sync(lbm_handle* h) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_set_graph_steps(lbm_handle* h, int steps_per_graph) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, steps_per_graph >= 0 && steps_per_graph % 2 == 0, LBM_ERR_ARG, "steps per graph must be even and >= 0");
    REQUIRE(h, h->persist == 0 || steps_per_graph % h->persist == 0, LBM_ERR_ARG,
            "steps per graph must be a multiple of the steps per persistent launch");
    drop_graph(h);
    h->graph_steps = steps_per_graph;
    return LBM_OK;
}

lbm_status lbm_set_persistent(lbm_handle* h, int steps_per_launch) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, steps_per_launch == 0 || (steps_per_launch >= 2 && steps_per_launch % 2 == 0), LBM_ERR_ARG,
            "steps per persistent launch must be 0 or even and >= 2");
    REQUIRE(h, steps_per_launch == 0 || h->graph_steps % steps_per_launch == 0, LBM_ERR_ARG,
            "steps per graph must be a multiple of the steps per persistent launch");
    CK(h, cudaSetDevice(h->d.device));
    if (steps_per_launch > 0 && !h->bar) {
        CK(h, cudaMalloc(&h->bar, 2 * sizeof(unsigned)));
        CK(h, cudaMemsetAsync(h->bar, 0, 2 * sizeof(unsigned), h->st));
    }
    drop_graph(h);
    h->persist = steps_per_launch;
    return LBM_OK;
}

lbm_status lbm_preset_barrier(lbm_handle* h, unsigned extra_arrivals) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->bar, LBM_ERR_STATE, "no persistent barrier: call lbm_set_persistent first");
    CK(h, cudaSetDevice(h->d.device));
    CK(h, cudaMemcpyAsync(h->bar + 1, &extra_arrivals, sizeof(unsigned), cudaMemcpyHostToDevice, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_preset_flags(lbm_handle* h, unsigned flags) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, (flags & ~(unsigned)(FLAG_NONFINITE | FLAG_BOUNDS)) == 0, LBM_ERR_ARG,
            "only LBM_FLAG_NONFINITE and LBM_FLAG_BOUNDS can be preset");
    CK(h, cudaSetDevice(h->d.device));
    CK(h, cudaMemcpyAsync(h->flags, &flags, sizeof(unsigned), cudaMemcpyHostToDevice, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_get_counts(lbm_handle* h, lbm_counts* out) {
    if (!h || !out) return fail(h, LBM_ERR_ARG, "null handle or output");
    *out = h->counts;
    out->steps = h->steps;
    out->device_bytes = (int64_t)h->geo_bytes;
    return LBM_OK;
}

lbm_status lbm_get_classes(lbm_handle* h, uint8_t* cls) {
    if (!h || !cls) return fail(h, LBM_ERR_ARG, "null handle or output");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    CK(h, cudaMemcpyAsync(cls, h->g.cls, h->npts, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_get_distributions(lbm_handle* h, double* f) {
    if (!h || !f) return fail(h, LBM_ERR_ARG, "null handle or output");
    CK(h, cudaSetDevice(h->d.device));
    int rc = readout(h, true);
    if (rc) return rc;
    CK(h, cudaMemcpyAsync(f, h->out_f, sizeof(double) * h->g.nact * h->d.Q, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

}  // extern "C"

namespace {

// rho and u of every active node into the staging buffer h->macro (rho [na],
// then u [3 na] after one padding entry), on the step stream.
int macro_to_staging(lbm_handle* h) {
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state: call lbm_init_equilibrium / lbm_set_geometry first");
    const int64_t na = h->g.nact;
    if (!h->macro) CK(h, dalloc(h, &h->macro, sizeof(double) * 4 * (na + 1)));
    int rc = wait_staging(h, 0);
    if (rc) return rc;
    // the read-out launch computes rho and u itself (no FP64 copy of f)
    StepParams p = make_params(h, 2);
    p.out_rho = h->macro;
    p.out_u = h->macro + (na + 1);
    CK(h, launch(h, 2, p));
    CK(h, reduce_partials(h->partials, h->nblocks, h->sums, h->st));
    return LBM_OK;
}

int macro_copies(lbm_handle* h, double* rho, double* u3, cudaStream_t st) {
    const int64_t na = h->g.nact;
    if (rho && na) CK(h, cudaMemcpyAsync(rho, h->macro, sizeof(double) * na, cudaMemcpyDeviceToHost, st));
    if (u3 && na)
        CK(h, cudaMemcpyAsync(u3, h->macro + (na + 1), sizeof(double) * 3 * na, cudaMemcpyDeviceToHost, st));
    return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_get_macro(lbm_handle* h, double* rho, double* u3) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    CK(h, cudaSetDevice(h->d.device));
    int rc = macro_to_staging(h);
    if (!rc) rc = macro_copies(h, rho, u3, h->st);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_get_macro_async(lbm_handle* h, double* rho, double* u3) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    CK(h, cudaSetDevice(h->d.device));
    int rc = ensure_copy_stream(h);
    if (!rc) rc = macro_to_staging(h);
    if (rc) return rc;
    CK(h, cudaEventRecord(h->ev_ready, h->st));
    CK(h, cudaStreamWaitEvent(h->cst, h->ev_ready, 0));
    rc = macro_copies(h, rho, u3, h->cst);
    if (rc) return rc;
    CK(h, cudaEventRecord(h->ev_copied[0], h->cst));
    return LBM_OK;
}

lbm_status lbm_wait_outputs(lbm_handle* h) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    CK(h, cudaSetDevice(h->d.device));
    if (h->cst) CK(h, cudaStreamSynchronize(h->cst));
    return LBM_OK;
}

}  // extern "C"

namespace {

// FP32 stress ring: folded steps are in the accumulators; the last step
// m = steps - 1 was preceded by a fold at step f = m - m % kFoldEvery (of
// the kFoldEvery steps before f), so steps f .. m, ring slots f % kRingSlots
// .. m % kRingSlots, are pending; |tau| of step m is in slot `last`.
void ring_pending(const lbm_handle* h, int& first, int& pending, int& last) {
    first = 0; pending = 0; last = -1;
    if (h->steps > 0) {
        const int64_t m = h->steps - 1;
        last = (int)(m % kRingSlots);
        pending = (int)(m % kFoldEvery) + 1;
        first = last - pending + 1;
    }
}

// Next-to-wall accumulators as doubles: |tau| (n), tau (3n, [3][n]), |tau| sum (n).
int read_accumulators(lbm_handle* h, std::vector<double>& w, std::vector<double>& a, std::vector<double>& am) {
    const int64_t n = h->g.nnw;
    w.assign(n, 0.0); a.assign(3 * n, 0.0); am.assign(n, 0.0);
    if (!n) return LBM_OK;
    if (h->d.precision == LBM_F64) {
        CK(h, cudaMemcpyAsync(w.data(), h->nw_wss, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaMemcpyAsync(a.data(), h->nw_acc, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaMemcpyAsync(am.data(), h->nw_accm, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaStreamSynchronize(h->st));
        return LBM_OK;
    }
    int first, pending, last;
    ring_pending(h, first, pending, last);
    if (!h->nw_out) CK(h, dalloc(h, &h->nw_out, sizeof(double) * 5 * n));
    CK(h, nw_readout_f32(h->nw_accf, h->nw_ring, n, first, pending, last, h->wss_from_ckpt ? h->nw_wssf : nullptr,
                         h->nw_out, h->st));
    CK(h, cudaMemcpyAsync(w.data(), h->nw_out, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaMemcpyAsync(a.data(), h->nw_out + n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaMemcpyAsync(am.data(), h->nw_out + 4 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

int write_accumulators(lbm_handle* h, const std::vector<double>& w, const std::vector<double>& a,
                       const std::vector<double>& am) {
    const int64_t n = h->g.nnw;
    if (!n) return LBM_OK;
    if (h->d.precision == LBM_F64) {
        CK(h, cudaMemcpyAsync(h->nw_wss, w.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->st));
        CK(h, cudaMemcpyAsync(h->nw_acc, a.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->st));
        CK(h, cudaMemcpyAsync(h->nw_accm, am.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->st));
        CK(h, cudaStreamSynchronize(h->st));
        return LBM_OK;
    }
    std::vector<float> wf(n);
    std::vector<float2> af(4 * n);
    auto split = [](double v) { float hi = (float)v; return make_float2(hi, (float)(v - (double)hi)); };
    for (int64_t p = 0; p < n; ++p) {
        wf[p] = (float)w[p];
        for (int c = 0; c < 3; ++c) af[c * n + p] = split(a[c * n + p]);
        af[3 * n + p] = split(am[p]);
    }
    CK(h, cudaMemcpyAsync(h->nw_wssf, wf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, h->st));
    CK(h, cudaMemcpyAsync(h->nw_accf, af.data(), sizeof(float2) * 4 * n, cudaMemcpyHostToDevice, h->st));
    // the accumulators hold every step so far: no ring slot is pending
    CK(h, cudaMemsetAsync(h->nw_ring, 0, sizeof(float) * kRingSlots * 4 * (n + 1), h->st));
    h->wss_from_ckpt = true;
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// Next-to-wall outputs [wss | normal n x 3 | acc n x 3 | acc_mag | osi | tawss]
// assembled in the staging buffer h->nw_fields, on the step stream.
int wss_to_staging(lbm_handle* h) {
    const int64_t n = h->g.nnw;
    int rc = wait_staging(h, 1);
    if (rc) return rc;
    const double *w, *a, *am;
    if (h->d.precision == LBM_F64) {
        w = h->nw_wss; a = h->nw_acc; am = h->nw_accm;
    } else {
        int first, pending, last;
        ring_pending(h, first, pending, last);
        if (!h->nw_out) CK(h, dalloc(h, &h->nw_out, sizeof(double) * 5 * n));
        CK(h, nw_readout_f32(h->nw_accf, h->nw_ring, n, first, pending, last,
                             h->wss_from_ckpt ? h->nw_wssf : nullptr, h->nw_out, h->st));
        w = h->nw_out; a = h->nw_out + n; am = h->nw_out + 4 * n;
    }
    if (!h->nw_fields) CK(h, dalloc(h, &h->nw_fields, sizeof(double) * 10 * n));
    CK(h, wss_outputs(w, a, am, h->nw_n, n, h->d.tawss_div, h->nw_fields, h->st));
    return LBM_OK;
}

int wss_copies(lbm_handle* h, int64_t* pt, double* normal3, double* wss, double* acc3, double* acc_mag, double* osi,
               double* tawss, cudaStream_t st) {
    const int64_t n = h->g.nnw;
    const double* o = h->nw_fields;
    const size_t b1 = sizeof(double) * n, b3 = 3 * b1;
    if (pt) CK(h, cudaMemcpyAsync(pt, h->g.nw_pt, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st));
    if (wss) CK(h, cudaMemcpyAsync(wss, o, b1, cudaMemcpyDeviceToHost, st));
    if (normal3) CK(h, cudaMemcpyAsync(normal3, o + n, b3, cudaMemcpyDeviceToHost, st));
    if (acc3) CK(h, cudaMemcpyAsync(acc3, o + 4 * n, b3, cudaMemcpyDeviceToHost, st));
    if (acc_mag) CK(h, cudaMemcpyAsync(acc_mag, o + 7 * n, b1, cudaMemcpyDeviceToHost, st));
    if (osi) CK(h, cudaMemcpyAsync(osi, o + 8 * n, b1, cudaMemcpyDeviceToHost, st));
    if (tawss) CK(h, cudaMemcpyAsync(tawss, o + 9 * n, b1, cudaMemcpyDeviceToHost, st));
    return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_get_wss(lbm_handle* h, int64_t* pt, double* normal3, double* wss, double* acc3, double* acc_mag,
                       double* osi, double* tawss) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    CK(h, cudaSetDevice(h->d.device));
    if (h->g.nnw == 0) return LBM_OK;
    // accumulators as doubles on the device, the outputs assembled there and
    // copied straight into the caller's buffers
    int rc = wss_to_staging(h);
    if (!rc) rc = wss_copies(h, pt, normal3, wss, acc3, acc_mag, osi, tawss, h->st);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
    return LBM_OK;
}

lbm_status lbm_get_wss_async(lbm_handle* h, int64_t* pt, double* normal3, double* wss, double* acc3,
                             double* acc_mag, double* osi, double* tawss) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    CK(h, cudaSetDevice(h->d.device));
    if (h->g.nnw == 0) return LBM_OK;
    int rc = ensure_copy_stream(h);
    if (!rc) rc = wss_to_staging(h);
    if (rc) return rc;
    CK(h, cudaEventRecord(h->ev_ready, h->st));
    CK(h, cudaStreamWaitEvent(h->cst, h->ev_ready, 0));
    rc = wss_copies(h, pt, normal3, wss, acc3, acc_mag, osi, tawss, h->cst);
    if (rc) return rc;
    CK(h, cudaEventRecord(h->ev_copied[1], h->cst));
    return LBM_OK;
}

lbm_status lbm_nearest_next_to_wall(lbm_handle* h, const double* xyz, int64_t nv, int max_radius, int64_t* nw_index,
                                    double* distance) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the geometry first");
    REQUIRE(h, nv >= 0 && (nv == 0 || (xyz && nw_index)), LBM_ERR_ARG, "null points or output");
    REQUIRE(h, max_radius >= 1 && max_radius <= 1024, LBM_ERR_ARG, "max_radius must be in [1, 1024]");
    if (nv == 0) return LBM_OK;
    CK(h, cudaSetDevice(h->d.device));
    double *d_xyz = nullptr, *d_dist = nullptr;
    int64_t* d_idx = nullptr;
    CK(h, cudaMalloc(&d_xyz, sizeof(double) * 3 * nv));
    cudaError_t e = cudaMalloc(&d_idx, sizeof(int64_t) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&d_dist, sizeof(double) * nv);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = nearest_next_to_wall(d_xyz, nv, h->g, h->nx, h->ny, h->nz, h->d.origin, h->d.spacing, max_radius, d_idx,
                                 d_dist, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nw_index, d_idx, sizeof(int64_t) * nv, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess && distance)
        e = cudaMemcpyAsync(distance, d_dist, sizeof(double) * nv, cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(d_xyz);
    if (d_idx) cudaFree(d_idx);
    if (d_dist) cudaFree(d_dist);
    if (e != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("nearest_next_to_wall: ") + cudaGetErrorString(e));
    return LBM_OK;
}

lbm_status lbm_get_conservation(lbm_handle* h, double* mass, double* mom3, double* flux) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    CK(h, cudaSetDevice(h->d.device));
    int rc = readout(h, false);
    if (rc) return rc;
    double s[kPartialStride];
    CK(h, cudaMemcpyAsync(s, h->sums, sizeof(s), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (mass) *mass = (double)h->g.nact + s[0];  // the kernel sums rho - 1
    if (mom3) { mom3[0] = s[1]; mom3[1] = s[2]; mom3[2] = s[3]; }
    if (flux) {
        // per-entry flux of the boundary-condition nodes, summed per rule in list order
        std::vector<double> fx(h->g.nsp);
        if (h->g.nsp) CK(h, cudaMemcpyAsync(fx.data(), h->sp_flux, sizeof(double) * h->g.nsp,
                                            cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaStreamSynchronize(h->st));
        for (int b = 0; b < h->nbc; ++b) flux[b] = 0.0;
        for (int64_t e = 0; e < h->g.nsp; ++e)
            if (h->sp_bc[e] >= 0 && h->sp_bc[e] < h->nbc) flux[h->sp_bc[e]] += fx[e];
    }
    return LBM_OK;
}

lbm_status lbm_save(lbm_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBM_ERR_ARG, "null handle or path");
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state to save");
    const int64_t na = h->g.nact, nn = h->g.nnw;
    std::vector<double> f(na * h->d.Q), acc, accm, wss;
    int rc = lbm_get_distributions(h, f.data());
    if (rc) return rc;
    rc = read_accumulators(h, wss, acc, accm);
    if (rc) return rc;
    std::FILE* fp = std::fopen(path, "wb");
    REQUIRE(h, fp, LBM_ERR_IO, std::string("cannot write ") + path);
    const uint32_t head[2] = {kCkptMagic, kCkptVersion};
    const int32_t cfg[6] = {h->d.Q, h->d.precision, h->d.mode, h->nx, h->ny, h->nz};
    const int64_t sz[4] = {na, nn, h->steps, (int64_t)h->waves.size()};
    std::vector<int64_t> wl;
    for (const auto& w : h->waves) wl.push_back((int64_t)w.size());
    bool ok = std::fwrite(head, sizeof(head), 1, fp) == 1 && std::fwrite(cfg, sizeof(cfg), 1, fp) == 1 &&
              std::fwrite(sz, sizeof(sz), 1, fp) == 1 &&
              std::fwrite(f.data(), sizeof(double), f.size(), fp) == f.size() &&
              std::fwrite(acc.data(), sizeof(double), acc.size(), fp) == acc.size() &&
              std::fwrite(accm.data(), sizeof(double), accm.size(), fp) == accm.size() &&
              std::fwrite(wss.data(), sizeof(double), wss.size(), fp) == wss.size() &&
              std::fwrite(wl.data(), sizeof(int64_t), wl.size(), fp) == wl.size();
    for (const auto& w : h->waves)
        ok = ok && (w.empty() || std::fwrite(w.data(), sizeof(double), w.size(), fp) == w.size());
    ok = (std::fclose(fp) == 0) && ok;
    REQUIRE(h, ok, LBM_ERR_IO, std::string("short write to ") + path);
    return LBM_OK;
}

lbm_status lbm_load(lbm_handle* h, const char* path) {
    if (!h || !path) return fail(h, LBM_ERR_ARG, "null handle or path");
    REQUIRE(h, h->has_geo, LBM_ERR_STATE, "set the same geometry before loading");
    std::FILE* fp = std::fopen(path, "rb");
    REQUIRE(h, fp, LBM_ERR_IO, std::string("cannot open ") + path);
    uint32_t head[2];
    int32_t cfg[6];
    int64_t sz[4];
    bool ok = std::fread(head, sizeof(head), 1, fp) == 1 && std::fread(cfg, sizeof(cfg), 1, fp) == 1 &&
              std::fread(sz, sizeof(sz), 1, fp) == 1;
    if (!ok || head[0] != kCkptMagic || head[1] != kCkptVersion) {
        std::fclose(fp);
        return fail(h, LBM_ERR_IO, "not a checkpoint of this version");
    }
    if (cfg[0] != h->d.Q || cfg[3] != h->nx || cfg[4] != h->ny || cfg[5] != h->nz || sz[0] != h->g.nact ||
        sz[1] != h->g.nnw || sz[3] < 1 || sz[3] > LBM_MAX_WAVES) {
        std::fclose(fp);
        return fail(h, LBM_ERR_ARG, "checkpoint lattice does not match this handle");
    }
    const int64_t na = sz[0], nn = sz[1];
    std::vector<double> f(na * h->d.Q), acc(3 * nn), accm(nn), wss(nn);
    std::vector<int64_t> wl(sz[3] <= LBM_MAX_WAVES ? sz[3] : 0);
    ok = sz[3] <= LBM_MAX_WAVES && std::fread(f.data(), sizeof(double), f.size(), fp) == f.size() &&
         std::fread(acc.data(), sizeof(double), acc.size(), fp) == acc.size() &&
         std::fread(accm.data(), sizeof(double), accm.size(), fp) == accm.size() &&
         std::fread(wss.data(), sizeof(double), wss.size(), fp) == wss.size() &&
         std::fread(wl.data(), sizeof(int64_t), wl.size(), fp) == wl.size();
    std::vector<std::vector<double>> waves(wl.size());
    for (size_t w = 0; ok && w < wl.size(); ++w) {
        ok = wl[w] >= 0 && wl[w] < ((int64_t)1 << 40);
        if (ok) {
            waves[w].resize(wl[w]);
            ok = waves[w].empty() || std::fread(waves[w].data(), sizeof(double), wl[w], fp) == (size_t)wl[w];
        }
    }
    std::fclose(fp);
    REQUIRE(h, ok, LBM_ERR_IO, std::string("truncated checkpoint ") + path);
    h->waves = waves;
    if (h->waves.empty()) h->waves.assign(1, std::vector<double>(1, 0.0));
    int rc = upload_waves(h);
    if (rc) return rc;
    rc = write_accumulators(h, wss, acc, accm);
    if (rc) return rc;
    h->steps = sz[2];
    return lbm_set_distributions(h, f.data());
}

lbm_status lbm_set_variant(lbm_handle* h, int variant) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, variant >= 0 && variant < kNumVariants, LBM_ERR_ARG, "variant out of range");
    drop_graph(h);
    h->variant = variant;
    return LBM_OK;
}

lbm_status lbm_autotune(lbm_handle* h, int trial_steps, int* best, float* ms_per_step) {
    if (!h) return fail(nullptr, LBM_ERR_ARG, "null handle");
    REQUIRE(h, h->has_state, LBM_ERR_STATE, "no state: set the geometry first");
    REQUIRE(h, trial_steps > 0, LBM_ERR_ARG, "trial_steps must be > 0");
    CK(h, cudaSetDevice(h->d.device));
    CK(h, cudaStreamSynchronize(h->st));
    // snapshot of everything a step writes, restored after every trial
    const size_t fbytes = (size_t)elem_size(h->d.precision) * h->d.Q * h->stride;
    const size_t rs = real_size(h->d.precision);
    struct Item { void* live; size_t bytes; void* copy; };
    std::vector<Item> items = {
        {h->buf[0], fbytes, nullptr}, {h->buf[1], fbytes, nullptr}, {h->slots, 2 * sizeof(int64_t), nullptr},
        {h->flags, sizeof(unsigned), nullptr},
        {h->nw_acc, sizeof(double) * 3 * (h->g.nnw + 1), nullptr},
        {h->nw_accm, sizeof(double) * (h->g.nnw + 1), nullptr},
        {h->nw_wss, sizeof(double) * (h->g.nnw + 1), nullptr},
        {h->nw_accf, sizeof(float2) * 4 * (h->g.nnw + 1), nullptr},
        {h->nw_wssf, sizeof(float) * (h->g.nnw + 1), nullptr},
        {h->nw_ring, sizeof(float) * kRingSlots * 4 * (h->g.nnw + 1), nullptr}};
    if (h->stale) items.push_back({h->stale, rs * h->d.Q * (h->g.nsp + 1), nullptr});
    if (h->nw_prev) items.push_back({h->nw_prev, rs * 4 * (h->g.nnw + 1), nullptr});
    auto release = [&]() {
        for (Item& it : items)
            if (it.copy) cudaFree(it.copy);
    };
    for (Item& it : items) {
        cudaError_t e = cudaMalloc(&it.copy, it.bytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it.copy, it.live, it.bytes, cudaMemcpyDeviceToDevice, h->st);
        if (e != cudaSuccess) {
            release();
            return fail(h, LBM_ERR_ALLOC, std::string("autotune snapshot: ") + cudaGetErrorString(e));
        }
    }
    const int64_t steps0 = h->steps, since0 = h->since_start, launches0 = h->launches;
    const int cur0 = h->cur, v0 = h->variant;
    auto restore = [&]() -> cudaError_t {
        for (Item& it : items) {
            cudaError_t e = cudaMemcpyAsync(it.live, it.copy, it.bytes, cudaMemcpyDeviceToDevice, h->st);
            if (e != cudaSuccess) return e;
        }
        h->steps = steps0; h->since_start = since0; h->cur = cur0;
        return cudaSuccess;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    int best_v = v0;
    cudaError_t err = cudaSuccess;
    for (int v = 0; v < kNumVariants && err == cudaSuccess; ++v) {
        err = restore();
        if (err != cudaSuccess) break;
        h->variant = v;
        for (int k = 0; k < 2 && err == cudaSuccess; ++k) {  // warm-up
            err = launch(h, 0, make_params(h, 0));
            h->cur ^= 1;
            h->steps++;
        }
        if (err != cudaSuccess) break;
        cudaEventRecord(e0, h->st);
        for (int k = 0; k < trial_steps && err == cudaSuccess; ++k) {
            err = launch(h, 0, make_params(h, 0));
            h->cur ^= 1;
            h->steps++;
        }
        cudaEventRecord(e1, h->st);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)trial_steps;
        if (ms_per_step) ms_per_step[v] = ms;
        if (err == cudaSuccess && ms < best_ms) { best_ms = ms; best_v = v; }
    }
    cudaError_t e2 = restore();
    if (err == cudaSuccess) err = e2;
    if (err == cudaSuccess) err = cudaStreamSynchronize(h->st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release();
    h->launches = launches0;
    h->variant = best_v;
    drop_graph(h);
    if (err != cudaSuccess) return fail(h, LBM_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(err));
    if (best) *best = best_v;
    return LBM_OK;
}

lbm_status lbm_get_stream(lbm_handle* h, void** stream) {
    if (!h || !stream) return fail(h, LBM_ERR_ARG, "null handle or output");
    *stream = (void*)h->st;
    return LBM_OK;
}

lbm_status lbm_get_launch_count(lbm_handle* h, int64_t* launches) {
    if (!h || !launches) return fail(h, LBM_ERR_ARG, "null handle or output");
    *launches = h->launches;
    return LBM_OK;
}

}  // extern "C"
