// C ABI of the octgb library (declared in include/octgb.h).
//
// The context owns one CUDA stream (or borrows the caller's), the uploaded
// geometry, grow-only device work buffers and the row accumulators.  Every
// entry point catches all C++ exceptions and reports failures as status codes
// plus a message; none of them exits the process.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <cstdio>
#include <exception>
#include <string>
#include <vector>
#include <cmath>
#include <algorithm>

#include "../../include/octgb.h"
#include "octgb_internal.h"

using namespace octgb;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    // once a captured graph may hold p, growing keeps the old allocation
    // alive (until release) instead of freeing it under the graph
    bool keep_old = false;
    std::vector<void*> retired;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) {
            if (keep_old) retired.push_back(p); else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        for (void* q : retired) cudaFree(q);
        retired.clear();
        p = nullptr;
        cap = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct Plan {
    int n_rows, r0, R, c0, C, n_out_z, n_tile_x, n_y;
    int cblk_first = 0, n_cblk = 0, xs_max = 1, rs_max = 1;
    std::vector<int2> zblk_h, cblk_h;   // host copies of the block tables
    bool lateral_identity = false;      // WxT is the identity (single-tile output grid)
    bool lateral_quad_local = false;    // every non-zero lateral weight stays inside the column's B-scan quad
    DevBuf zr, wz0, wz1, xr, wx0, wx1, fz, shift, lo, hi, zblk, cblk, zrow, zf, xcol;
    bool opc = false;
    StitchDev dev() const {
        StitchDev d;
        d.zr = zr.as<int>();
        d.wz0 = wz0.as<float>();
        d.wz1 = wz1.as<float>();
        d.xr = xr.as<int>();
        d.wx0 = wx0.as<float>();
        d.wx1 = wx1.as<float>();
        d.fz = fz.as<float>();
        d.shift = opc ? shift.as<int>() : nullptr;
        d.lo = opc ? lo.as<int>() : nullptr;
        d.hi = opc ? hi.as<int>() : nullptr;
        d.zblk = zblk.as<int2>();
        d.cblk = cblk.as<int2>();
        d.zrow = zrow.as<float4>();
        d.zf = zf.as<float2>();
        d.xcol = xcol.as<float4>();
        d.cblk_first = cblk_first;
        d.n_cblk = n_cblk;
        d.r0 = r0;
        d.R = R;
        d.c0 = c0;
        d.C = C;
        d.n_out_z = n_out_z;
        d.n_tile_x = n_tile_x;
        d.n_rows = n_rows;
        return d;
    }
    void release() {
        for (DevBuf* b : {&zr, &wz0, &wz1, &xr, &wx0, &wx1, &fz, &shift, &lo, &hi, &zblk, &cblk, &zrow, &zf, &xcol})
            b->release();
    }
};

// Which tiles touch each output block of the frame-batch stitch kernel, with
// their patch extents and shared-memory offsets; built once per tile list.
struct SlotTable {
    std::vector<int> key;        // plan ids, n_out_z, n_out_x, rows per block
    DevBuf slots, counts;
    size_t smem = 0;             // largest patch footprint of a block (bytes)
    int ns_max = 1;              // most tiles touching one block
    void release() {
        slots.release();
        counts.release();
    }
};

// A device tile table of the batched form.  A graph captured over a batch
// call holds the table's address, so a table is never overwritten once a
// capture used it (pinned); unpinned tables are recycled least recently used.
struct QTable {
    std::vector<QueueTile> key;  // the uploaded contents
    uint64_t hash = 0;           // FNV-1a of the contents, compared before the bytes
    DevBuf buf;
    bool pinned = false;
    uint64_t last_use = 0;
};

struct Error : std::exception {
    int code;
    std::string msg;
    Error(int c, std::string m) : code(c), msg(std::move(m)) {}
};

std::string g_create_error;

}  // namespace

struct octgb_ctx {
    int device = 0;
    int num_sms = 0;
    int stitch_rows = kStitchRows;           // frame-batch stitch block height (octgb_set_stitch_rows)
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    std::atomic<int> cancel{0};
    std::atomic<int64_t> launches{0};
    // geometry
    bool has_geom = false;
    int taps = 0;
    int U = 0;
    DevBuf w, start, win, tw, wsh, s0;
    // work buffers
    DevBuf raw, apod, out, mm, frames;
    int* status_host = nullptr;  // mapped pinned status word
    int* status_dev = nullptr;
    // plans and row state
    std::vector<Plan*> plans;
    DevBuf plan_table;           // device array of StitchDev, one per plan
    int xs_max = 1, rs_max = 1;  // largest stitch patch over all plans
    DevBuf run_mm;               // running [min, max] (ordered uint) of finite dB
    std::vector<cudaGraphExec_t> graphs;
    std::vector<int64_t> graph_kernels;
    bool capturing = false;
    int64_t capture_launch0 = 0;
    DevBuf magbuf, dbbuf, planemm, segs, qtable;
    DevBuf qcounter;                         // batched form: queue head
    // legacy TIFF encoding
    DevBuf enc_bits, enc_lut, enc_slots, enc_sizes;
    // rare raw formats: prepared batch, frame-mean lines, per-file magnitudes
    DevBuf prep, prep_apod, magrep, srr, gemm_part;
    // precision form (tensor-core sinc)
    bool prec_ok = false;
    DevBuf prec_w, prec_kb, prec_hi, prec_lo, prec_m, prec_x;
    // float64 form: band weights (tap-major), window / N and twiddles in float64
    DevBuf ex_w, ex_win, ex_tw;
    DevBuf bias_part;                        // CNN training: per-plane sums of the bias gradient
    DevBuf wgrad_part;                       // CNN training: per-CTA sums of the tensor-core weight gradient
    // dispersion scorer and focus profiles
    bool win_is_one = false;                 // geometry window is exactly 1 (plain linearisation)
    DevBuf disp_x, disp_hann, disp_phase, disp_a, disp_score, xmed;
    int disp_b = 0, disp_rep = 0, disp_nx = 0;
    std::vector<double> dk2;
    std::vector<QTable*> qtables;            // batched form: device tile tables by content
    uint64_t qtable_clock = 0;
    std::vector<SlotTable*> slot_tables;
    // host-input staging of the frame API: a copy stream and a ring of device
    // slots, so the copy of one batch overlaps the kernels of the previous one
    static constexpr int kRing = 3;
    cudaStream_t copy = nullptr;
    DevBuf ring[kRing];
    cudaEvent_t ring_ready[kRing] = {nullptr, nullptr, nullptr};
    cudaEvent_t ring_free[kRing] = {nullptr, nullptr, nullptr};
    int ring_next = 0;
    DevBuf num, den;
    int row_nf = 0, row_nz = 0, row_nx = 0;
    bool row_open = false;
};

namespace {

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(OCTGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void require(bool ok, const char* msg) {
    if (!ok) throw Error(OCTGB_ERR_ARG, msg);
}

template <typename F>
int guarded(octgb_ctx* ctx, F&& f) {
    if (ctx == nullptr) return OCTGB_ERR_ARG;
    try {
        ck(cudaSetDevice(ctx->device), "cudaSetDevice");
        f();
        ctx->err.clear();
        return OCTGB_OK;
    } catch (const Error& e) {
        ctx->err = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        ctx->err = "host allocation failed";
        return OCTGB_ERR_NOMEM;
    } catch (const std::exception& e) {
        ctx->err = e.what();
        return OCTGB_ERR_STATE;
    } catch (...) {
        ctx->err = "unknown error";
        return OCTGB_ERR_STATE;
    }
}

size_t raw_elem(int dtype) { return dtype == OCTGB_F32 ? 4 : 2; }

// Make the raw batch available on the device; returns the device pointer.
const void* stage_raw(octgb_ctx* c, const void* raw, int dtype, int loc, size_t bytes) {
    if (loc == OCTGB_DEVICE) return raw;
    ck(c->raw.ensure(bytes), "cudaMalloc(raw)");
    ck(cudaMemcpyAsync(c->raw.p, raw, bytes, cudaMemcpyHostToDevice, c->stream), "H2D raw");
    return c->raw.p;
}

void check_status(octgb_ctx* c) {
    if (c->capturing) throw Error(OCTGB_ERR_STATE, "a host-synchronising call was made during graph capture");
    ck(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    const int s = *reinterpret_cast<volatile int*>(c->status_host);
    if (s != kStatusOk) {
        *reinterpret_cast<volatile int*>(c->status_host) = kStatusOk;
        throw Error(OCTGB_ERR_TIMEOUT, "a bounded device-side wait expired (bulk copy did not complete)");
    }
}

void validate_raw(const void* raw, int dtype, int loc, int B, int interf, int apod) {
    require(raw != nullptr, "raw is NULL");
    require(dtype == OCTGB_U16 || dtype == OCTGB_I16 || dtype == OCTGB_F32, "raw_dtype must be U16, I16 or F32");
    require(loc == OCTGB_HOST || loc == OCTGB_DEVICE, "bad location flag");
    require(B >= 0, "B < 0");
    require(apod >= 1 && apod < 32768, "apod_size must be in [1, 32767]");
    require(interf > apod, "interf must exceed apod_size");
    if (loc == OCTGB_DEVICE) require((reinterpret_cast<uintptr_t>(raw) & 15u) == 0, "device raw must be 16-byte aligned");
}

// Launch apod mean + fused spectral kernel over n_seg device batches (same B, interf, apod).
void launch_spectral_segs(octgb_ctx* c, const void* const* segs, int n_seg, int dtype, int B, int interf, int apod,
                          int mode, float* out_dev, int z0, int nz, unsigned int* mm_dev,
                          const double* hann = nullptr, const float2* hann2 = nullptr) {
    if (B == 0 || n_seg == 0) return;
    ck(c->apod.ensure(static_cast<size_t>(n_seg) * B * kN * sizeof(float) + 16), "cudaMalloc(apod)");
    SpectralArgs a{};
    a.raw = segs[0];
    for (int i = 0; i < n_seg; ++i) a.seg[i] = segs[i];
    a.n_seg = n_seg;
    a.B = B;
    a.interf = interf;
    a.apod = apod;
    a.nx = interf - apod;
    a.n_ascans = static_cast<int64_t>(n_seg) * B * (interf - apod);
    a.apod_mean = c->apod.as<float>();
    a.g.w = c->w.as<float>();
    a.g.start = c->start.as<int>();
    a.g.taps = c->taps;
    a.g.win = c->win.as<float2>();
    a.g.tw = c->tw.as<float2>();
    a.g.wsh = c->wsh.as<float>();
    a.g.s0 = c->s0.as<int>();
    a.g.U = c->U;
    a.out = out_dev;
    a.z0 = z0;
    a.nz = nz;
    a.minmax = mm_dev;
    a.hann = hann;
    a.hann2 = hann2;
    a.status = c->status_dev;
    ck(launch_apod_mean(a, dtype, c->stream), "apod kernel");
    c->launches++;
    const int64_t pairs = (a.n_ascans + kPerCta - 1) / kPerCta;
    int64_t grid = static_cast<int64_t>(c->num_sms) * spectral_max_ctas_per_sm(dtype, mode);
    if (grid > pairs) grid = pairs;
    if (grid < 1) return;
    ck(launch_spectral(a, dtype, mode, static_cast<int>(grid), c->stream), "spectral kernel");
    c->launches++;
}

// Run the spectral stage of a batch into `out` (device) in the given mode.
void run_spectral(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod, int mode,
                  float* out_dev, int z0, int nz, unsigned int* mm_dev, const double* hann = nullptr,
                  const float2* hann2 = nullptr) {
    if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
    if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
    if (B == 0) return;  // empty batch: nothing to launch
    const size_t bytes = static_cast<size_t>(B) * interf * kN * raw_elem(dtype);
    const void* rd = stage_raw(c, raw, dtype, loc, bytes);
    launch_spectral_segs(c, &rd, 1, dtype, B, interf, apod, mode, out_dev, z0, nz, mm_dev, hann, hann2);
}

void copy_out(octgb_ctx* c, void* dst, int loc, const void* src_dev, size_t bytes) {
    if (bytes == 0) return;
    ck(cudaMemcpyAsync(dst, src_dev, bytes, loc == OCTGB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       c->stream),
       "copy out");
}

void read_minmax(octgb_ctx* c, const unsigned int* mm_dev, double* out2) {
    unsigned int h[2];
    ck(cudaMemcpyAsync(h, mm_dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "D2H minmax");
    check_status(c);
    if (h[0] == 0xffffffffu) {
        out2[0] = out2[1] = NAN;
    } else {
        out2[0] = ord2f(h[0]);
        out2[1] = ord2f(h[1]);
    }
}

const SlotTable& slot_table(octgb_ctx* c, int n_tiles, const int* plan_ids, int n_out_z, int n_out_x, int rows) {
    std::vector<int> key(plan_ids, plan_ids + n_tiles);
    key.push_back(n_out_z);
    key.push_back(n_out_x);
    key.push_back(rows);
    for (SlotTable* t : c->slot_tables)
        if (t->key == key) return *t;
    require(!c->capturing, "first use of a tile list during graph capture: run the sequence once before capturing");
    const int nxb = (n_out_x + kBlk - 1) / kBlk, nzb = (n_out_z + rows - 1) / rows;
    std::vector<StitchSlot> slots(static_cast<size_t>(nxb) * nzb * n_tiles);
    std::vector<int> counts(static_cast<size_t>(nxb) * nzb, 0);
    size_t smem = 0;
    int ns_max = 1;
    for (int bz = 0; bz < nzb; ++bz) {
        for (int bx = 0; bx < nxb; ++bx) {
            const int blk = bz * nxb + bx;
            int n = 0, off = 0;
            for (int t = 0; t < n_tiles; ++t) {
                const Plan& p = *c->plans[plan_ids[t]];
                const int cbi = bx - p.cblk_first;
                if (cbi < 0 || cbi >= p.n_cblk || p.cblk_h[cbi].x < 0) continue;
                int lo = 1 << 30, hi = -1;
                for (int k = bz * (rows / kBlk); k < (bz + 1) * (rows / kBlk); ++k) {
                    if (k >= static_cast<int>(p.zblk_h.size()) || p.zblk_h[k].x < 0) continue;
                    lo = lo < p.zblk_h[k].x ? lo : p.zblk_h[k].x;
                    hi = hi > p.zblk_h[k].y ? hi : p.zblk_h[k].y;
                }
                if (hi < 0) continue;
                StitchSlot s{};
                s.t = t;
                s.x_lo = p.cblk_h[cbi].x;
                s.xs = p.cblk_h[cbi].y - p.cblk_h[cbi].x + 1;
                s.r_lo = lo;
                s.rs = hi - lo + 1;
                s.off = off;
                s.opc = p.opc ? 1 : 0;
                // one zero row after each A-scan's rows and one zero A-scan after the
                // last, so the kernel's 2 x 2 reads need no bounds tests; an odd
                // stride puts neighbouring A-scans in different banks
                s.rst = (s.rs + 1) | 1;
                off += (s.xs + 1) * s.rst * (p.opc ? 2 : 1);
                slots[static_cast<size_t>(blk) * n_tiles + n++] = s;
            }
            counts[blk] = n;
            ns_max = ns_max > n ? ns_max : n;
            smem = smem > static_cast<size_t>(off) * sizeof(float) ? smem : static_cast<size_t>(off) * sizeof(float);
        }
    }
    require(smem <= 160 * 1024, "stitch patches of one output block exceed shared memory");
    SlotTable* t = new SlotTable();
    t->key = key;
    t->smem = smem;
    t->ns_max = ns_max;
    try {
        ck(t->slots.ensure(slots.size() * sizeof(StitchSlot) + 16), "cudaMalloc(slots)");
        ck(t->counts.ensure(counts.size() * sizeof(int) + 16), "cudaMalloc(slot counts)");
        ck(cudaMemcpyAsync(t->slots.p, slots.data(), slots.size() * sizeof(StitchSlot), cudaMemcpyHostToDevice,
                           c->stream),
           "H2D slots");
        ck(cudaMemcpyAsync(t->counts.p, counts.data(), counts.size() * sizeof(int), cudaMemcpyHostToDevice,
                           c->stream),
           "H2D slot counts");
        ck(cudaStreamSynchronize(c->stream), "sync slot table");
    } catch (...) {
        t->release();
        delete t;
        throw;
    }
    c->slot_tables.push_back(t);
    return *t;
}

// The device copy of a batched-form tile table.  Tables are kept by content:
// a batch repeated with the same tiles reuses its table, a table used while a
// graph is captured is pinned (the graph replays with its address), and at
// most kMaxFreeTables unpinned tables (16 KiB each) are kept, the least
// recently used one being overwritten (in stream order, after every kernel
// that read it): a sequence of up to that many distinct batches (one per tile,
// say) can be run once and then captured.
constexpr int kMaxFreeTables = 128;

uint64_t fnv1a(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

const QueueTile* tile_table(octgb_ctx* c, const std::vector<QueueTile>& qt) {
    const size_t bytes = qt.size() * sizeof(QueueTile);
    const uint64_t hash = fnv1a(qt.data(), bytes);
    ++c->qtable_clock;
    for (QTable* t : c->qtables)
        if (t->hash == hash && t->key.size() == qt.size() && memcmp(t->key.data(), qt.data(), bytes) == 0) {
            t->last_use = c->qtable_clock;
            if (c->capturing) t->pinned = true;
            return t->buf.as<QueueTile>();
        }
    require(!c->capturing, "first use of a tile table during graph capture: run the batch once first");
    QTable* t = nullptr;
    int n_free = 0;
    for (QTable* u : c->qtables)
        if (!u->pinned) {
            ++n_free;
            if (t == nullptr || u->last_use < t->last_use) t = u;
        }
    if (n_free < kMaxFreeTables) {
        t = new QTable();
        c->qtables.push_back(t);
    }
    t->key.clear();                       // a failed upload leaves no matching entry
    ck(t->buf.ensure(static_cast<size_t>(kMaxQueueTiles) * sizeof(QueueTile)), "cudaMalloc(tile table)");
    t->key = qt;
    t->hash = hash;
    t->last_use = c->qtable_clock;
    // from pageable memory: the call returns once the source is staged
    ck(cudaMemcpyAsync(t->buf.p, t->key.data(), bytes, cudaMemcpyHostToDevice, c->stream), "H2D tile table");
    return t->buf.as<QueueTile>();
}

}  // namespace

extern "C" {

int octgb_create(int device, octgb_ctx** out) {
    if (out == nullptr) return OCTGB_ERR_ARG;
    *out = nullptr;
    octgb_ctx* c = nullptr;
    try {
        c = new octgb_ctx();
        c->device = device;
        ck(cudaSetDevice(device), "cudaSetDevice");
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        if (prop.major * 10 + prop.minor < 100)
            throw Error(OCTGB_ERR_STATE, std::string("device ") + prop.name + " is not sm_100 or newer");
        c->num_sms = prop.multiProcessorCount;
        // a blocking stream: ordered with the legacy default stream, on which
        // callers such as torch's default stream produce and read buffers
        ck(cudaStreamCreateWithFlags(&c->own, cudaStreamDefault), "cudaStreamCreate");
        c->stream = c->own;
        ck(cudaHostAlloc(reinterpret_cast<void**>(&c->status_host), sizeof(int), cudaHostAllocMapped),
           "cudaHostAlloc(status)");
        *c->status_host = kStatusOk;
        ck(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->status_dev), c->status_host, 0),
           "cudaHostGetDevicePointer");
        ck(c->mm.ensure(4096), "cudaMalloc(minmax)");
        *out = c;
        g_create_error.clear();
        return OCTGB_OK;
    } catch (const Error& e) {
        g_create_error = e.msg;
        if (c) octgb_destroy(c);
        return e.code;
    } catch (...) {
        g_create_error = "octgb_create failed";
        if (c) octgb_destroy(c);
        return OCTGB_ERR_STATE;
    }
}

int octgb_destroy(octgb_ctx* c) {
    if (c == nullptr) return OCTGB_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (Plan* p : c->plans) {
        if (p) {
            p->release();
            delete p;
        }
    }
    for (DevBuf* b : {&c->w, &c->start, &c->win, &c->tw, &c->wsh, &c->s0, &c->raw, &c->apod, &c->out, &c->mm, &c->frames, &c->num,
                      &c->den, &c->plan_table, &c->run_mm, &c->magbuf, &c->dbbuf, &c->planemm, &c->segs, &c->qtable,
                      &c->qcounter, &c->disp_x, &c->disp_hann, &c->disp_phase, &c->disp_a, &c->disp_score, &c->xmed,
                      &c->prec_w, &c->prec_kb, &c->prec_hi, &c->prec_lo, &c->prec_m, &c->prec_x, &c->ex_w, &c->ex_win, &c->ex_tw, &c->bias_part, &c->wgrad_part, &c->prep,
                      &c->prep_apod, &c->magrep, &c->srr, &c->gemm_part, &c->enc_bits, &c->enc_lut, &c->enc_slots, &c->enc_sizes})
        b->release();
    for (QTable* t : c->qtables) {
        t->buf.release();
        delete t;
    }
    for (cudaGraphExec_t g : c->graphs)
        if (g) cudaGraphExecDestroy(g);
    for (SlotTable* t : c->slot_tables) {
        t->release();
        delete t;
    }
    if (c->copy) cudaStreamSynchronize(c->copy);
    for (int k = 0; k < octgb_ctx::kRing; ++k) {
        c->ring[k].release();
        if (c->ring_ready[k]) cudaEventDestroy(c->ring_ready[k]);
        if (c->ring_free[k]) cudaEventDestroy(c->ring_free[k]);
    }
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->status_host) cudaFreeHost(c->status_host);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return OCTGB_OK;
}

const char* octgb_last_error(const octgb_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int octgb_set_stream(octgb_ctx* c, void* s) {
    return guarded(c, [&] { c->stream = s ? static_cast<cudaStream_t>(s) : c->own; });
}

int octgb_synchronize(octgb_ctx* c) {
    return guarded(c, [&] { check_status(c); });
}

int octgb_cancel(octgb_ctx* c) {
    if (!c) return OCTGB_ERR_ARG;
    c->cancel.store(1);
    return OCTGB_OK;
}

int octgb_reset_cancel(octgb_ctx* c) {
    if (!c) return OCTGB_ERR_ARG;
    c->cancel.store(0);
    return OCTGB_OK;
}

int64_t octgb_launch_count(const octgb_ctx* c) { return c ? c->launches.load() : 0; }

int octgb_set_geometry(octgb_ctx* c, int n, int taps, const int64_t* idx, const double* w, const double* window) {
    return guarded(c, [&] {
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry during graph capture");
        if (!c->graphs.empty())
            throw Error(OCTGB_ERR_STATE,
                        "the context holds captured graphs that replay its current geometry: "
                        "call octgb_graphs_release before setting a new geometry");
        require(n == kN, "n must be 2048");
        require(taps >= 1 && taps <= kMaxTaps, "taps must be in [1, 32]");
        require(idx && w && window, "NULL geometry array");
        std::vector<float> wt(static_cast<size_t>(taps) * kN);
        std::vector<int> st(kN);
        for (int i = 0; i < kN; ++i) {
            int s = -1;
            for (int t = 0; t < taps; ++t) {
                const double wv = w[static_cast<size_t>(i) * taps + t];
                const int64_t j = idx[static_cast<size_t>(i) * taps + t];
                require(j >= 0 && j < kN, "sinc index out of range");
                if (t == 0) s = static_cast<int>(j);
                const bool pad_entry = (wv == 0.0 && j == 0 && t > 0);
                if (!pad_entry) require(j == s + t, "sinc taps of a row must be contiguous increasing indices");
                wt[static_cast<size_t>(t) * kN + i] = static_cast<float>(wv);
            }
            st[i] = s;
        }
        // shifted dense weights of the spectral kernel: thread t owns outputs
        // 4t..4t+3 and reads the U source samples s0_t .. s0_t + U - 1; at step u
        // it reads the one congruent to u (mod U), so wsh[t][r][u] = weight of
        // source s0_t + v, (s0_t + v) = u (mod U), for output 4t + r.  With
        // gcd(U, 32) = 2 the samples a warp reads at one step are U apart (or
        // the same sample): distinct banks of a linear line.
        std::vector<int> len(kN, 0);
        for (int i = 0; i < kN; ++i) {
            for (int t = 0; t < taps; ++t)
                if (!(t > 0 && idx[static_cast<size_t>(i) * taps + t] == 0)) len[i] = t + 1;
        }
        int U_need = 0;
        for (int t = 0; t < kThreads; ++t) {
            const int base = st[4 * t];
            for (int r = 0; r < 4; ++r) {
                const int i = 4 * t + r;
                require(st[i] >= base, "sinc band starts must not decrease");
                const int reach = st[i] - base + len[i];
                U_need = U_need > reach ? U_need : reach;
            }
        }
        int U = U_need <= 14 ? 14 : (U_need <= 18 ? 18 : (U_need <= 22 ? 22 : (U_need <= 26 ? 26 : 0)));
        require(U > 0, "sinc band too wide for the spectral kernel (4 outputs need > 26 source samples)");
        std::vector<float> wsh(static_cast<size_t>(kThreads) * 4 * U, 0.f);
        std::vector<int> s0v(kThreads);
        for (int t = 0; t < kThreads; ++t) {
            const int base = st[4 * t];
            s0v[t] = base;
            for (int r = 0; r < 4; ++r) {
                const int i = 4 * t + r;
                for (int k = 0; k < len[i]; ++k) {
                    const int u = (st[i] + k) % U;         // step that reads source st[i] + k
                    wsh[(static_cast<size_t>(t) * 4 + r) * U + u] = wt[static_cast<size_t>(k) * kN + i];
                }
            }
        }
        std::vector<float2> win(kN), tw(kN);
        for (int i = 0; i < kN; ++i) {
            // complex64 window (core/spectral.py:219) times 1/N: exact power-of-two scaling
            win[i] = make_float2(static_cast<float>(window[2 * i]) * (1.0f / kN),
                                 static_cast<float>(window[2 * i + 1]) * (1.0f / kN));
            const double ang = 2.0 * 3.14159265358979323846 * i / kN;
            tw[i] = make_float2(static_cast<float>(cos(ang)), static_cast<float>(sin(ang)));
        }
        ck(c->w.ensure(wt.size() * sizeof(float)), "cudaMalloc(w)");
        ck(c->start.ensure(kN * sizeof(int)), "cudaMalloc(start)");
        ck(c->win.ensure(kN * sizeof(float2)), "cudaMalloc(win)");
        ck(c->tw.ensure(kN * sizeof(float2)), "cudaMalloc(tw)");
        ck(cudaMemcpyAsync(c->w.p, wt.data(), wt.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream), "H2D w");
        ck(cudaMemcpyAsync(c->start.p, st.data(), kN * sizeof(int), cudaMemcpyHostToDevice, c->stream), "H2D start");
        ck(cudaMemcpyAsync(c->win.p, win.data(), kN * sizeof(float2), cudaMemcpyHostToDevice, c->stream), "H2D win");
        ck(cudaMemcpyAsync(c->tw.p, tw.data(), kN * sizeof(float2), cudaMemcpyHostToDevice, c->stream), "H2D tw");
        ck(c->wsh.ensure(wsh.size() * sizeof(float)), "cudaMalloc(wsh)");
        ck(c->s0.ensure(s0v.size() * sizeof(int)), "cudaMalloc(s0)");
        ck(cudaMemcpyAsync(c->wsh.p, wsh.data(), wsh.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream),
           "H2D wsh");
        ck(cudaMemcpyAsync(c->s0.p, s0v.data(), s0v.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream),
           "H2D s0");
        // float64 form: the band weights as given (tap-major), window / N and twiddles in float64
        {
            std::vector<double> wd(static_cast<size_t>(taps) * kN, 0.0);
            std::vector<double2> wind(kN), twd(kN);
            for (int i = 0; i < kN; ++i) {
                for (int t = 0; t < len[i]; ++t) wd[static_cast<size_t>(t) * kN + i] = w[static_cast<size_t>(i) * taps + t];
                wind[i] = make_double2(window[2 * i] * (1.0 / kN), window[2 * i + 1] * (1.0 / kN));
                const double ang = 2.0 * 3.14159265358979323846 * i / kN;
                twd[i] = make_double2(cos(ang), sin(ang));
            }
            ck(c->ex_w.ensure(wd.size() * sizeof(double)), "cudaMalloc(float64 weights)");
            ck(c->ex_win.ensure(kN * sizeof(double2)), "cudaMalloc(float64 window)");
            ck(c->ex_tw.ensure(kN * sizeof(double2)), "cudaMalloc(float64 twiddles)");
            ck(cudaMemcpyAsync(c->ex_w.p, wd.data(), wd.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream),
               "H2D float64 weights");
            ck(cudaMemcpyAsync(c->ex_win.p, wind.data(), kN * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
               "H2D float64 window");
            ck(cudaMemcpyAsync(c->ex_tw.p, twd.data(), kN * sizeof(double2), cudaMemcpyHostToDevice, c->stream),
               "H2D float64 twiddles");
            ck(cudaStreamSynchronize(c->stream), "sync float64 geometry");
        }
        // tensor-core sinc tiles of the precision form (when every output block's band fits its window)
        std::vector<uint16_t> ptiles;
        std::vector<int> pkb;
        c->prec_ok = build_prec_tiles(st.data(), len.data(), wt.data(), ptiles, pkb);
        if (c->prec_ok) {
            ck(c->prec_w.ensure(ptiles.size() * sizeof(uint16_t)), "cudaMalloc(precision tiles)");
            ck(c->prec_kb.ensure(pkb.size() * sizeof(int)), "cudaMalloc(precision windows)");
            ck(cudaMemcpyAsync(c->prec_w.p, ptiles.data(), ptiles.size() * sizeof(uint16_t), cudaMemcpyHostToDevice,
                               c->stream),
               "H2D precision tiles");
            ck(cudaMemcpyAsync(c->prec_kb.p, pkb.data(), pkb.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream),
               "H2D precision windows");
        }
        ck(cudaStreamSynchronize(c->stream), "sync geometry");
        c->U = U;
        c->taps = taps;
        c->has_geom = true;
        c->win_is_one = true;
        for (int i = 0; i < kN; ++i)
            if (window[2 * i] != 1.0 || window[2 * i + 1] != 0.0) c->win_is_one = false;
    });
}

int octgb_fused_pre_fft(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod, float* spec,
                        int spec_loc) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(spec != nullptr, "spec is NULL");
        const size_t ob = static_cast<size_t>(B) * (interf - apod) * kN * 2 * sizeof(float);
        float* dst = spec;
        if (spec_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(ob), "cudaMalloc(out)");
            dst = c->out.as<float>();
        }
        run_spectral(c, raw, dtype, loc, B, interf, apod, kModeSpec, dst, 0, 0, nullptr);
        if (spec_loc != OCTGB_DEVICE) copy_out(c, spec, OCTGB_HOST, dst, ob);
        check_status(c);
    });
}

int octgb_magnitude(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod, float* mag,
                    int mag_loc) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(mag != nullptr, "mag is NULL");
        const size_t ob = static_cast<size_t>(B) * (interf - apod) * kHalf * sizeof(float);
        float* dst = mag;
        if (mag_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(ob), "cudaMalloc(out)");
            dst = c->out.as<float>();
        }
        run_spectral(c, raw, dtype, loc, B, interf, apod, kModeMag, dst, 0, 0, nullptr);
        if (mag_loc != OCTGB_DEVICE) copy_out(c, mag, OCTGB_HOST, dst, ob);
        if (mag_loc != OCTGB_DEVICE || loc != OCTGB_DEVICE) check_status(c);
    });
}

int octgb_db(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod, int z0, int nz,
             float* db, int db_loc, double* minmax) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(db != nullptr, "db is NULL");
        require(z0 >= 0 && nz >= 1 && z0 + nz <= kHalf, "depth crop must lie within [0, N/2)");
        const size_t ob = static_cast<size_t>(B) * (interf - apod) * nz * sizeof(float);
        float* dst = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(ob), "cudaMalloc(out)");
            dst = c->out.as<float>();
        }
        unsigned int* mm = c->mm.as<unsigned int>();
        if (minmax) {
            ck(launch_minmax_init(mm, 2, c->stream), "minmax init");
            c->launches++;
        }
        run_spectral(c, raw, dtype, loc, B, interf, apod, kModeDb, dst, z0, nz, minmax ? mm : nullptr);
        if (db_loc != OCTGB_DEVICE) copy_out(c, db, OCTGB_HOST, dst, ob);
        if (minmax)
            read_minmax(c, mm, minmax);
        else if (db_loc != OCTGB_DEVICE || loc != OCTGB_DEVICE)
            check_status(c);
    });
}

int octgb_quantise(octgb_ctx* c, const float* db, int64_t n, int db_loc, double c1, double c2, uint16_t* bits,
                   int bits_loc) {
    return guarded(c, [&] {
        require(n >= 0, "n < 0");
        require(db && bits, "NULL array");
        if (c1 > c2) {
            const double t = c1;
            c1 = c2;
            c2 = t;
        }
        require(c2 > c1, "clim must span a non-empty range");
        const float* src = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->raw.ensure(static_cast<size_t>(n) * sizeof(float)), "cudaMalloc(db in)");
            ck(cudaMemcpyAsync(c->raw.p, db, static_cast<size_t>(n) * sizeof(float), cudaMemcpyHostToDevice,
                               c->stream),
               "H2D db");
            src = c->raw.as<float>();
        }
        uint16_t* dst = bits;
        if (bits_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(static_cast<size_t>(n) * sizeof(uint16_t)), "cudaMalloc(bits)");
            dst = c->out.as<uint16_t>();
        }
        ck(c->qtable.ensure(kQuantTable * sizeof(float)), "cudaMalloc(quant table)");
        ck(launch_quantise(src, n, c1, c2, c->qtable.as<float>(), dst, c->stream), "quantise kernel");
        c->launches += 2;
        if (bits_loc != OCTGB_DEVICE) {
            copy_out(c, bits, OCTGB_HOST, dst, static_cast<size_t>(n) * sizeof(uint16_t));
            check_status(c);
        }
    });
}

int octgb_minmax(octgb_ctx* c, const float* db, int64_t n, int db_loc, double* minmax) {
    return guarded(c, [&] {
        require(n >= 0 && db && minmax, "bad argument");
        const float* src = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->raw.ensure(static_cast<size_t>(n) * sizeof(float) + 16), "cudaMalloc(db in)");
            ck(cudaMemcpyAsync(c->raw.p, db, static_cast<size_t>(n) * sizeof(float), cudaMemcpyHostToDevice,
                               c->stream),
               "H2D db");
            src = c->raw.as<float>();
        }
        unsigned int* mm = c->mm.as<unsigned int>();
        ck(launch_minmax_init(mm, 2, c->stream), "minmax init");
        ck(launch_minmax(src, n, mm, c->stream), "minmax kernel");
        c->launches += 2;
        read_minmax(c, mm, minmax);
    });
}

int octgb_stitch_plan(octgb_ctx* c, int n_rows, int r0, int r1, int c0, int c1, int n_out_z, int n_tile_x,
                      const double* Wz, const double* WxT, const double* fz, const int64_t* shift, const double* pdz,
                      int n_y, int* plan_id) {
    return guarded(c, [&] {
        require(plan_id != nullptr, "plan_id is NULL");
        require(n_rows == kHalf, "n_rows must be N/2 = 1024");
        require(r0 >= 0 && r1 > r0 && r1 <= n_rows, "bad row window");
        require(c0 >= 0 && c1 > c0, "bad column window");
        require(n_out_z >= 1 && n_tile_x >= 2, "bad output / tile size");
        require(Wz && WxT && fz, "NULL operator");
        require((shift == nullptr) == (pdz == nullptr), "shift and pdz go together");
        const int R = r1 - r0, C = c1 - c0;
        // compact the depth operator: <= 2 adjacent non-zeros per output row
        std::vector<int> zr(n_out_z, -1), xr(C, -1);
        std::vector<float> wz0(n_out_z, 0.f), wz1(n_out_z, 0.f), wx0(C, 0.f), wx1(C, 0.f), fzf(R);
        for (int zo = 0; zo < n_out_z; ++zo) {
            int first = -1, last = -1;
            for (int r = 0; r < R; ++r) {
                if (Wz[static_cast<size_t>(zo) * R + r] != 0.0) {
                    if (first < 0) first = r;
                    last = r;
                }
            }
            if (first < 0) continue;
            require(last - first <= 1, "Wz row has more than two adjacent non-zeros");
            if (first == R - 1) first = R - 2 >= 0 ? R - 2 : 0;  // keep zr+1 inside the window
            zr[zo] = first;
            wz0[zo] = static_cast<float>(Wz[static_cast<size_t>(zo) * R + first]);
            wz1[zo] = first + 1 < R ? static_cast<float>(Wz[static_cast<size_t>(zo) * R + first + 1]) : 0.f;
        }
        for (int cc = 0; cc < C; ++cc) {
            int first = -1, last = -1;
            for (int x = 0; x < n_tile_x; ++x) {
                if (WxT[static_cast<size_t>(x) * C + cc] != 0.0) {
                    if (first < 0) first = x;
                    last = x;
                }
            }
            if (first < 0) continue;
            require(last - first <= 1, "WxT column has more than two adjacent non-zeros");
            if (first == n_tile_x - 1) first = n_tile_x - 2;
            xr[cc] = first;
            wx0[cc] = static_cast<float>(WxT[static_cast<size_t>(first) * C + cc]);
            wx1[cc] = static_cast<float>(WxT[static_cast<size_t>(first + 1) * C + cc]);
        }
        for (int r = 0; r < R; ++r) fzf[r] = static_cast<float>(fz[r]);
        // per 32 x 32 output block: the input rows / A-scans it reads (patch extents)
        const int nzb = (n_out_z + kBlk - 1) / kBlk;
        std::vector<int2> zb(nzb, make_int2(-1, -1));
        int rs_max = 1, xs_max = 1;
        for (int b = 0; b < nzb; ++b) {
            int lo = 1 << 30, hi = -1;
            for (int zo = b * kBlk; zo < n_out_z && zo < (b + 1) * kBlk; ++zo) {
                if (zr[zo] < 0) continue;
                lo = lo < zr[zo] ? lo : zr[zo];
                const int h = zr[zo] + 1 < R ? zr[zo] + 1 : R - 1;
                hi = hi > h ? hi : h;
            }
            if (hi >= 0) {
                zb[b] = make_int2(lo, hi);
                rs_max = rs_max > hi - lo + 1 ? rs_max : hi - lo + 1;
            }
        }
        const int cbf = c0 / kBlk, cbl = (c0 + C - 1) / kBlk;
        std::vector<int2> cbt(cbl - cbf + 1, make_int2(-1, -1));
        for (int b = cbf; b <= cbl; ++b) {
            int lo = 1 << 30, hi = -1;
            for (int cabs = b * kBlk; cabs < (b + 1) * kBlk; ++cabs) {
                const int cc = cabs - c0;
                if (cc < 0 || cc >= C || xr[cc] < 0) continue;
                lo = lo < xr[cc] ? lo : xr[cc];
                hi = hi > xr[cc] + 1 ? hi : xr[cc] + 1;
            }
            if (hi >= 0) {
                cbt[b - cbf] = make_int2(lo, hi);
                xs_max = xs_max > hi - lo + 1 ? xs_max : hi - lo + 1;
            }
        }
        require(static_cast<size_t>(2 * xs_max * rs_max + 2 * xs_max * kBlk) * sizeof(float) <= 160 * 1024,
                "stitch patch too large (output pixel much coarser than the tile sampling)");
        Plan* p = new Plan();
        p->lateral_identity = c0 == 0 && C == n_tile_x;
        // batched form: every quad holding output column cc must also hold the
        // A-scans it reads (xr with weight wx0, xr + 1 with wx1); quads start
        // at multiples of 4, the last one of a B-scan at C - 4
        p->lateral_quad_local = c0 == 0 && C == n_tile_x;
        const int qpb = (C + kPerCta - 1) / kPerCta;
        for (int qb = 0; qb < qpb && p->lateral_quad_local; ++qb) {
            const int q0 = (qb == qpb - 1 && C >= kPerCta) ? C - kPerCta : qb * kPerCta;
            for (int cc = q0; cc < q0 + kPerCta && cc < C; ++cc) {
                const bool ok0 = wx0[cc] == 0.f || (xr[cc] >= q0 && xr[cc] < q0 + kPerCta && xr[cc] < C);
                const bool ok1 = wx1[cc] == 0.f || (xr[cc] + 1 >= q0 && xr[cc] + 1 < q0 + kPerCta && xr[cc] + 1 < C);
                if (xr[cc] < 0 || !ok0 || !ok1) p->lateral_quad_local = false;
            }
        }
        p->zblk_h = zb;
        p->cblk_h = cbt;
        p->cblk_first = cbf;
        p->n_cblk = cbl - cbf + 1;
        p->xs_max = xs_max;
        p->rs_max = rs_max;
        p->n_rows = n_rows;
        p->r0 = r0;
        p->R = R;
        p->c0 = c0;
        p->C = C;
        p->n_out_z = n_out_z;
        p->n_tile_x = n_tile_x;
        p->n_y = n_y;
        auto up = [&](DevBuf& b, const void* src, size_t bytes) {
            ck(b.ensure(bytes > 0 ? bytes : 4), "cudaMalloc(plan)");
            if (bytes) ck(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream), "H2D plan");
        };
        try {
            up(p->zr, zr.data(), zr.size() * sizeof(int));
            up(p->wz0, wz0.data(), wz0.size() * sizeof(float));
            up(p->wz1, wz1.data(), wz1.size() * sizeof(float));
            up(p->xr, xr.data(), xr.size() * sizeof(int));
            up(p->wx0, wx0.data(), wx0.size() * sizeof(float));
            up(p->wx1, wx1.data(), wx1.size() * sizeof(float));
            up(p->fz, fzf.data(), fzf.size() * sizeof(float));
            up(p->zblk, zb.data(), zb.size() * sizeof(int2));
            up(p->cblk, cbt.data(), cbt.size() * sizeof(int2));
            // per output row, for the batched form's depth resampling: {zr, w0,
            // w1, d} and the focus weights {F[zr], F[zr + 1] (0 past the window)},
            // d = fma(F1, w1, F0 w0) as the kernel forms it
            std::vector<float4> zrow(n_out_z);
            std::vector<float2> zfv(n_out_z);
            for (int zo = 0; zo < n_out_z; ++zo) {
                const int z = zr[zo];
                const float f0 = z >= 0 ? fzf[z] : 0.f;
                const float f1 = z >= 0 && z + 1 < R ? fzf[z + 1] : 0.f;
                const float prod = f0 * wz0[zo];
                float zrf;
                memcpy(&zrf, &z, sizeof(float));
                zrow[zo] = make_float4(zrf, wz0[zo], wz1[zo], std::fmaf(f1, wz1[zo], prod));
                zfv[zo] = make_float2(f0, f1);
            }
            up(p->zrow, zrow.data(), zrow.size() * sizeof(float4));
            up(p->zf, zfv.data(), zfv.size() * sizeof(float2));
            // per output column: {xr (int bits), wx0, wx1, 0}
            std::vector<float4> xcol(C);
            for (int cc = 0; cc < C; ++cc) {
                float xrf;
                memcpy(&xrf, &xr[cc], sizeof(float));
                xcol[cc] = make_float4(xrf, wx0[cc], wx1[cc], 0.f);
            }
            up(p->xcol, xcol.data(), xcol.size() * sizeof(float4));
            if (shift != nullptr) {
                require(n_y >= 1, "n_y must be >= 1 with optical-path correction");
                const size_t m = static_cast<size_t>(n_y) * n_tile_x;
                std::vector<int> sh(m), lo(m), hi(m);
                for (size_t i = 0; i < m; ++i) {
                    sh[i] = static_cast<int>(shift[i]);
                    // exact integer form of 0 <= r + pdz <= n_rows - 1
                    lo[i] = static_cast<int>(ceil(-pdz[i]));
                    hi[i] = static_cast<int>(floor(n_rows - 1 - pdz[i]));
                }
                up(p->shift, sh.data(), m * sizeof(int));
                up(p->lo, lo.data(), m * sizeof(int));
                up(p->hi, hi.data(), m * sizeof(int));
                p->opc = true;
            }
            ck(cudaStreamSynchronize(c->stream), "sync plan");
        } catch (...) {
            p->release();
            delete p;
            throw;
        }
        c->plans.push_back(p);
        *plan_id = static_cast<int>(c->plans.size() - 1);
        // refresh the device plan table and the context-wide patch bound
        std::vector<StitchDev> table;
        for (Plan* q : c->plans) table.push_back(q->dev());
        ck(c->plan_table.ensure(table.size() * sizeof(StitchDev)), "cudaMalloc(plan table)");
        ck(cudaMemcpyAsync(c->plan_table.p, table.data(), table.size() * sizeof(StitchDev), cudaMemcpyHostToDevice,
                           c->stream),
           "H2D plan table");
        ck(cudaStreamSynchronize(c->stream), "sync plan table");
        c->xs_max = c->xs_max > xs_max ? c->xs_max : xs_max;
        c->rs_max = c->rs_max > rs_max ? c->rs_max : rs_max;
    });
}

int octgb_row_begin(octgb_ctx* c, int n_frames, int n_out_z, int n_out_x) {
    return guarded(c, [&] {
        require(n_frames >= 0 && n_out_z >= 1 && n_out_x >= 1, "bad row shape");
        const size_t bytes = static_cast<size_t>(n_frames) * n_out_z * n_out_x * sizeof(float);
        ck(c->num.ensure(bytes + 16), "cudaMalloc(num)");
        ck(c->den.ensure(bytes + 16), "cudaMalloc(den)");
        ck(cudaMemsetAsync(c->num.p, 0, bytes, c->stream), "memset num");
        ck(cudaMemsetAsync(c->den.p, 0, bytes, c->stream), "memset den");
        c->row_nf = n_frames;
        c->row_nz = n_out_z;
        c->row_nx = n_out_x;
        c->row_open = true;
    });
}

}  // extern "C"

namespace {
// TileStitcher.contribute of B frames of magnitudes (device, (B, n_tile_x,
// N/2)) into the row accumulators (pipeline.py:283-285)
void stitch_row(octgb_ctx* c, const Plan& p, const float* mag, const std::vector<int>& fy, bool contiguous, int B,
                int frame_offset) {
    const int* fdev = nullptr;
    if (!contiguous) {
        // pageable copy: returns once staged, so `fy` may go out of scope
        ck(c->frames.ensure(fy.size() * sizeof(int)), "cudaMalloc(frames)");
        ck(cudaMemcpyAsync(c->frames.p, fy.data(), fy.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream),
           "H2D frames");
        fdev = c->frames.as<int>();
    }
    ck(launch_stitch(p.dev(), mag, fdev, fy[0], B, c->num.as<float>(), c->den.as<float>(), frame_offset, c->row_nx,
                     p.xs_max, p.rs_max, c->stream),
       "stitch kernel");
    c->launches++;
}

// PrepArgs of a raw batch (prepare_raw, core/spectral.py:48-68); false when
// the batch needs no preparation (apodisation lines, no binning)
bool prep_args(PrepArgs& a, const void* raw, int B, int n_lines, int apod, int binning, int mode, int group) {
    require(binning >= 1 && binning <= 64, "AScanBinning must be in [1, 64]");
    require(mode == 0 || mode == 1, "apod_mode must be 0 (lines) or 1 (frame mean)");
    require(group >= 1 && B % group == 0, "the batch is not a whole number of frames (apod_group)");
    if (mode == 0) require(apod >= 1 && apod < n_lines, "apod_size must be in [1, lines)");
    a.raw = raw;
    a.B = B;
    a.n_lines = n_lines;
    a.mode = mode;
    a.group = group;
    a.binning = binning;
    a.a_out = mode == 0 ? apod : 1;
    a.scan0 = mode == 0 ? apod : 0;
    a.n_scan = n_lines - a.scan0;
    a.s0 = std::max(1, binning / 2) - 1;
    a.left = (binning + 1) / 2 - 1;
    a.n_kept = binning == 1 ? a.n_scan : (a.n_scan - a.s0 + binning - 1) / binning;
    require(a.n_kept >= 1, "no A-lines left after AScanBinning");
    return binning > 1 || mode == 1;
}

// prepared batch on the device (c->prep, float32 (B, a_out + n_kept, N))
void run_prepare(octgb_ctx* c, const PrepArgs& a0, int dtype, int loc) {
    PrepArgs a = a0;
    const size_t bytes = static_cast<size_t>(a.B) * a.n_lines * kN * raw_elem(dtype);
    a.raw = stage_raw(c, a.raw, dtype, loc, bytes);
    ck(c->prep.ensure(static_cast<size_t>(a.B) * (a.a_out + a.n_kept) * kN * sizeof(float) + 16),
       "cudaMalloc(prepared)");
    if (a.mode == 1)
        ck(c->prep_apod.ensure(static_cast<size_t>(a.B / a.group) * kN * sizeof(float)), "cudaMalloc(frame mean)");
    ck(launch_prepare(a, dtype, c->prep_apod.as<float>(), c->prep.as<float>(), c->stream), "prepare kernel");
    c->launches += a.mode == 1 ? 2 : 1;
}
}  // namespace

extern "C" {

int octgb_row_add_batch(octgb_ctx* c, int plan_id, const void* raw, int dtype, int loc, int B, int interf, int apod,
                        const int64_t* frame_idx, int frame_offset) {
    return guarded(c, [&] {
        if (!c->row_open) throw Error(OCTGB_ERR_STATE, "octgb_row_begin has not been called");
        require(plan_id >= 0 && plan_id < static_cast<int>(c->plans.size()), "bad plan id");
        const Plan& p = *c->plans[plan_id];
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(interf - apod == p.n_tile_x, "A-scans per B-scan differ from the plan's tile width");
        require(p.n_out_z == c->row_nz && p.c0 + p.C <= c->row_nx, "plan does not fit the row");
        require(frame_offset >= 0 && frame_offset + B <= c->row_nf, "frames outside the row");
        require(frame_idx != nullptr, "frame_idx is NULL");
        std::vector<int> fy(B > 0 ? B : 1);
        bool contiguous = true;
        for (int f = 0; f < B; ++f) {
            require(!p.opc || (frame_idx[f] >= 0 && frame_idx[f] < p.n_y), "frame index outside the scan");
            fy[f] = static_cast<int>(frame_idx[f]);
            contiguous = contiguous && frame_idx[f] == frame_idx[0] + f;
        }
        if (B == 0) return;
        const size_t mb = static_cast<size_t>(B) * p.n_tile_x * kHalf * sizeof(float);
        ck(c->magbuf.ensure(mb), "cudaMalloc(mag)");
        run_spectral(c, raw, dtype, loc, B, interf, apod, kModeMag, c->magbuf.as<float>(), 0, 0, nullptr);
        stitch_row(c, p, c->magbuf.as<float>(), fy, contiguous, B, frame_offset);
    });
}

int octgb_row_finalise(octgb_ctx* c, float thr, float* db, int db_loc, double* plane_minmax) {
    return guarded(c, [&] {
        if (!c->row_open) throw Error(OCTGB_ERR_STATE, "octgb_row_begin has not been called");
        require(db != nullptr, "db is NULL");
        const int64_t per = static_cast<int64_t>(c->row_nz) * c->row_nx;
        const size_t bytes = static_cast<size_t>(c->row_nf) * per * sizeof(float);
        float* dst = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(bytes + 16), "cudaMalloc(db)");
            dst = c->out.as<float>();
        }
        unsigned int* mm = nullptr;
        DevBuf tmp;
        if (plane_minmax) {
            ck(c->mm.ensure(static_cast<size_t>(2 * c->row_nf) * sizeof(unsigned int) + 16), "cudaMalloc(mm)");
            mm = c->mm.as<unsigned int>();
            ck(launch_minmax_init(mm, 2 * c->row_nf, c->stream), "minmax init");
            c->launches++;
        }
        ck(launch_finalise(c->num.as<float>(), c->den.as<float>(), per, c->row_nf, thr, dst, mm, c->stream),
           "finalise kernel");
        c->launches++;
        if (db_loc != OCTGB_DEVICE) copy_out(c, db, OCTGB_HOST, dst, bytes);
        if (plane_minmax) {
            std::vector<unsigned int> h(2 * static_cast<size_t>(c->row_nf));
            ck(cudaMemcpyAsync(h.data(), mm, h.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream),
               "D2H plane minmax");
            check_status(c);
            for (int f = 0; f < c->row_nf; ++f) {
                if (h[2 * f] == 0xffffffffu) {
                    plane_minmax[2 * f] = plane_minmax[2 * f + 1] = NAN;
                } else {
                    plane_minmax[2 * f] = ord2f(h[2 * f]);
                    plane_minmax[2 * f + 1] = ord2f(h[2 * f + 1]);
                }
            }
        } else {
            check_status(c);
        }
        c->row_open = false;
    });
}


int octgb_frames_process(octgb_ctx* c, int n_tiles, const int* plan_ids, const void* const* raws, int dtype, int loc,
                         int B, int interf, int apod, int f0, int n_out_z, int n_out_x, float thr, float* db,
                         int db_loc, double* plane_minmax) {
    return guarded(c, [&] {
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        require(n_tiles >= 1 && n_tiles <= kMaxSeg, "n_tiles must be in [1, 32]");
        require(plan_ids && raws && db, "NULL argument");
        require(n_out_z >= 1 && n_out_x >= 1, "bad output shape");
        require(!(db_loc == OCTGB_HOST && c->capturing), "host output during graph capture");
        TileList tl{};
        tl.n = n_tiles;
        for (int t = 0; t < n_tiles; ++t) {
            require(plan_ids[t] >= 0 && plan_ids[t] < static_cast<int>(c->plans.size()), "bad plan id");
            const Plan& p = *c->plans[plan_ids[t]];
            require(p.n_tile_x == interf - apod, "A-scans per B-scan differ from a plan's tile width");
            require(p.n_out_z == n_out_z && p.c0 + p.C <= n_out_x, "a plan does not fit the output grid");
            require(!p.opc || (f0 >= 0 && f0 + B <= p.n_y), "frames outside the scan");
            validate_raw(raws[t], dtype, loc, B, interf, apod);
            tl.id[t] = plan_ids[t];
        }
        if (B == 0) return;
        const size_t tile_bytes = static_cast<size_t>(B) * interf * kN * raw_elem(dtype);
        const void* segs[kMaxSeg];
        int slot = -1;
        if (loc == OCTGB_HOST) {
            require(!c->capturing, "host input during graph capture");
            if (c->copy == nullptr) {
                ck(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking), "cudaStreamCreate(copy)");
                for (int k = 0; k < octgb_ctx::kRing; ++k) {
                    ck(cudaEventCreateWithFlags(&c->ring_ready[k], cudaEventDisableTiming), "cudaEventCreate");
                    ck(cudaEventCreateWithFlags(&c->ring_free[k], cudaEventDisableTiming), "cudaEventCreate");
                }
            }
            slot = c->ring_next;
            c->ring_next = (slot + 1) % octgb_ctx::kRing;
            ck(c->ring[slot].ensure(tile_bytes * n_tiles), "cudaMalloc(raw ring)");
            // the slot's previous batch must have left the spectral kernel
            ck(cudaStreamWaitEvent(c->copy, c->ring_free[slot], 0), "cudaStreamWaitEvent");
            for (int t = 0; t < n_tiles; ++t) {
                void* dst = static_cast<char*>(c->ring[slot].p) + t * tile_bytes;
                ck(cudaMemcpyAsync(dst, raws[t], tile_bytes, cudaMemcpyHostToDevice, c->copy), "H2D raw");
                segs[t] = dst;
            }
            ck(cudaEventRecord(c->ring_ready[slot], c->copy), "cudaEventRecord");
            ck(cudaStreamWaitEvent(c->stream, c->ring_ready[slot], 0), "cudaStreamWaitEvent");
        } else {
            for (int t = 0; t < n_tiles; ++t) segs[t] = raws[t];
        }
        const int nx = interf - apod;
        const int64_t tile_stride = static_cast<int64_t>(B) * nx * kHalf;
        ck(c->magbuf.ensure(static_cast<size_t>(tile_stride) * n_tiles * sizeof(float)), "cudaMalloc(mag)");
        launch_spectral_segs(c, segs, n_tiles, dtype, B, interf, apod, kModeMag, c->magbuf.as<float>(), 0, 0, nullptr);
        if (slot >= 0) ck(cudaEventRecord(c->ring_free[slot], c->stream), "cudaEventRecord");
        const size_t db_bytes = static_cast<size_t>(B) * n_out_z * n_out_x * sizeof(float);
        float* dst = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->dbbuf.ensure(db_bytes), "cudaMalloc(db)");
            dst = c->dbbuf.as<float>();
        }
        unsigned int* pmm = nullptr;
        if (plane_minmax) {
            require(!c->capturing, "per-plane clims are read on the host: not during graph capture");
            ck(c->planemm.ensure(static_cast<size_t>(2 * B) * sizeof(unsigned int)), "cudaMalloc(plane mm)");
            pmm = c->planemm.as<unsigned int>();
            ck(launch_minmax_init(pmm, 2 * B, c->stream), "minmax init");
            c->launches++;
        }
        ck(c->run_mm.ensure(2 * sizeof(unsigned int)), "cudaMalloc(run mm)");
        const SlotTable& stab = slot_table(c, n_tiles, plan_ids, n_out_z, n_out_x, c->stitch_rows);
        ck(launch_stitch_frames(c->plan_table.as<StitchDev>(), tl, stab.slots.as<StitchSlot>(), stab.counts.as<int>(),
                                stab.ns_max, stab.smem, c->magbuf.as<float>(), tile_stride, B, nx, f0, n_out_z, n_out_x, thr, dst,
                                pmm, c->run_mm.as<unsigned int>(), c->stitch_rows, c->stream),
           "stitch frames kernel");
        c->launches++;
        if (db_loc != OCTGB_DEVICE) copy_out(c, db, OCTGB_HOST, dst, db_bytes);
        if (plane_minmax) {
            std::vector<unsigned int> h(2 * static_cast<size_t>(B));
            ck(cudaMemcpyAsync(h.data(), pmm, h.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream),
               "D2H plane minmax");
            check_status(c);
            for (int f = 0; f < B; ++f) {
                const bool none = h[2 * f] == 0xffffffffu;
                plane_minmax[2 * f] = none ? NAN : ord2f(h[2 * f]);
                plane_minmax[2 * f + 1] = none ? NAN : ord2f(h[2 * f + 1]);
            }
        } else if (db_loc != OCTGB_DEVICE) {
            check_status(c);
        }
    });
}

int octgb_clim_reset(octgb_ctx* c) {
    return guarded(c, [&] {
        ck(c->run_mm.ensure(2 * sizeof(unsigned int)), "cudaMalloc(run mm)");
        ck(launch_minmax_init(c->run_mm.as<unsigned int>(), 2, c->stream), "minmax init");
        c->launches++;
    });
}

int octgb_clim_get(octgb_ctx* c, double* clim) {
    return guarded(c, [&] {
        require(clim != nullptr, "clim is NULL");
        ck(c->run_mm.ensure(2 * sizeof(unsigned int)), "cudaMalloc(run mm)");
        read_minmax(c, c->run_mm.as<unsigned int>(), clim);
    });
}

int octgb_quantise_running(octgb_ctx* c, const float* db, int64_t n, int db_loc, uint16_t* bits, int bits_loc) {
    return guarded(c, [&] {
        require(n >= 0 && db && bits, "bad argument");
        require(db_loc == OCTGB_DEVICE && bits_loc == OCTGB_DEVICE, "octgb_quantise_running takes device arrays");
        ck(c->run_mm.ensure(2 * sizeof(unsigned int)), "cudaMalloc(run mm)");
        ck(c->qtable.ensure(kQuantTable * sizeof(float)), "cudaMalloc(quant table)");
        ck(launch_quantise_dev(db, n, c->run_mm.as<unsigned int>(), c->qtable.as<float>(), bits, c->stream),
           "quantise kernel");
        c->launches += 2;
    });
}

int octgb_graph_begin(octgb_ctx* c) {
    return guarded(c, [&] {
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "already capturing");
        ck(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
        c->capturing = true;
        c->capture_launch0 = c->launches.load();
    });
}

int octgb_graph_end(octgb_ctx* c, int* graph_id) {
    return guarded(c, [&] {
        if (!c->capturing) throw Error(OCTGB_ERR_STATE, "not capturing");
        require(graph_id != nullptr, "graph_id is NULL");
        c->capturing = false;
        cudaGraph_t g = nullptr;
        ck(cudaStreamEndCapture(c->stream, &g), "cudaStreamEndCapture");
        cudaGraphExec_t ge = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        ck(e, "cudaGraphInstantiate");
        c->graphs.push_back(ge);
        c->graph_kernels.push_back(c->launches.load() - c->capture_launch0);
        // the graph holds the addresses of the context's buffers: from now on
        // a buffer that grows keeps its old allocation until octgb_destroy
        for (DevBuf* b : {&c->raw, &c->apod, &c->out, &c->mm, &c->frames, &c->num, &c->den, &c->plan_table,
                          &c->run_mm, &c->magbuf, &c->dbbuf, &c->planemm, &c->segs, &c->qtable, &c->qcounter,
                          &c->disp_x, &c->disp_hann, &c->disp_phase, &c->disp_a, &c->disp_score, &c->xmed,
                          &c->prec_hi, &c->prec_lo, &c->prec_m, &c->prec_x, &c->prep, &c->prep_apod,
                          &c->magrep, &c->srr, &c->gemm_part, &c->enc_bits, &c->enc_lut, &c->enc_slots, &c->enc_sizes})
            b->keep_old = true;
        for (int k = 0; k < octgb_ctx::kRing; ++k) c->ring[k].keep_old = true;
        c->launches.store(c->capture_launch0);
        *graph_id = static_cast<int>(c->graphs.size() - 1);
    });
}

int octgb_graph_launch(octgb_ctx* c, int graph_id) {
    return guarded(c, [&] {
        require(graph_id >= 0 && graph_id < static_cast<int>(c->graphs.size()) && c->graphs[graph_id],
                "bad graph id");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        ck(cudaGraphLaunch(c->graphs[graph_id], c->stream), "cudaGraphLaunch");
        c->launches += c->graph_kernels[graph_id];
    });
}


int octgb_graphs_release(octgb_ctx* c) {
    return guarded(c, [&] {
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "octgb_graphs_release during graph capture");
        ck(cudaStreamSynchronize(c->stream), "sync before graph release");
        for (cudaGraphExec_t g : c->graphs)
            if (g) cudaGraphExecDestroy(g);
        c->graphs.clear();
        c->graph_kernels.clear();
        for (QTable* t : c->qtables) t->pinned = false;
    });
}

int octgb_set_stitch_rows(octgb_ctx* c, int rows) {
    return guarded(c, [&] {
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "octgb_set_stitch_rows during graph capture");
        require(rows == 32 || rows == 64 || rows == 128, "stitch rows must be 32, 64 or 128");
        c->stitch_rows = rows;
    });
}

int octgb_batch_process(octgb_ctx* c, int n_tiles, const octgb_tile* tiles, int dtype, float thr, int grab) {
    return guarded(c, [&] {
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        require(n_tiles >= 1 && n_tiles <= kMaxQueueTiles, "n_tiles must be in [1, 256]");
        require(tiles != nullptr, "tiles is NULL");
        require(grab >= 1 && grab <= 4096, "grab must be in [1, 4096]");
        std::vector<QueueTile> qt(n_tiles);
        unsigned int quads = 0;
        int rows = 0;
        for (int t = 0; t < n_tiles; ++t) {
            const octgb_tile& d = tiles[t];
            validate_raw(d.raw, dtype, OCTGB_DEVICE, d.B, d.interf, d.apod_size);
            require(d.db != nullptr, "tile db is NULL");
            require(d.plan_id >= 0 && d.plan_id < static_cast<int>(c->plans.size()), "bad plan id");
            const Plan& p = *c->plans[d.plan_id];
            require(p.n_tile_x == d.interf - d.apod_size, "A-scans per B-scan differ from the tile's plan");
            require(p.lateral_quad_local,
                    "a batched tile's plan must be a single-tile plan (output columns = the tile's A-scans)");
            require(!p.opc, "the batched form does not take optical-path correction");
            require(p.n_out_z <= 1600, "the batched form resamples to at most 1600 output rows per A-scan");
            const int qpb = (d.interf - d.apod_size + kPerCta - 1) / kPerCta;
            const unsigned int nq = static_cast<unsigned int>(static_cast<int64_t>(d.B) * qpb);
            require(static_cast<uint64_t>(quads) + nq < (1ull << 31), "batch too large");
            QueueTile& q = qt[t];
            q.raw = d.raw;
            q.out = d.db;
            q.plan = c->plan_table.as<StitchDev>() + d.plan_id;
            q.B = d.B;
            q.interf = d.interf;
            q.apod = d.apod_size;
            q.nx = d.interf - d.apod_size;
            q.nz = p.n_out_z;
            q.apod_row0 = rows;
            q.quad0 = quads;
            q.nquads = nq;
            q.qpb = qpb;
            quads += nq;
            rows += d.B;
        }
        if (quads == 0) return;
        const QueueTile* qdev = tile_table(c, qt);
        ck(c->apod.ensure(static_cast<size_t>(rows) * kN * sizeof(float) + 16), "cudaMalloc(apod)");
        ck(c->qcounter.ensure(sizeof(unsigned int)), "cudaMalloc(queue head)");
        ck(c->run_mm.ensure(2 * sizeof(unsigned int)), "cudaMalloc(run mm)");
        ck(cudaMemsetAsync(c->qcounter.p, 0, sizeof(unsigned int), c->stream), "memset queue head");
        ck(launch_apod_mean_tiles(qdev, n_tiles, rows, dtype, c->apod.as<float>(), c->stream),
           "apod kernel");
        c->launches++;
        SpectralArgs a{};
        a.n_seg = 1;
        a.B = 1;
        a.nx = 1;
        a.apod_mean = c->apod.as<float>();
        a.g.w = c->w.as<float>();
        a.g.start = c->start.as<int>();
        a.g.taps = c->taps;
        a.g.win = c->win.as<float2>();
        a.g.tw = c->tw.as<float2>();
        a.g.wsh = c->wsh.as<float>();
        a.g.s0 = c->s0.as<int>();
        a.g.U = c->U;
        a.minmax = c->run_mm.as<unsigned int>();
        a.status = c->status_dev;
        a.qt = qdev;
        a.n_qt = n_tiles;
        a.counter = c->qcounter.as<unsigned int>();
        a.total_quads = quads;
        a.grab = grab;
        a.thr = thr;
        int64_t grid = static_cast<int64_t>(c->num_sms) * spectral_max_ctas_per_sm(dtype, kModeResample);
        if (grid > quads) grid = quads;
        ck(launch_spectral(a, dtype, kModeResample, static_cast<int>(grid), c->stream), "spectral kernel");
        c->launches++;
    });
}

// ---------------------------------------------------------------------------
// Dispersion scorer (octrecon/estimation/dispersion.py:66-107) and focus
// depth profiles (octrecon/estimation/focus.py:146,156,255).

int octgb_disp_load(octgb_ctx* c, const void* raw, int dtype, int loc, int n_bscans, int rep, int interf, int apod,
                    const double* hann) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, n_bscans, interf, apod);
        require(c->has_geom && c->win_is_one,
                "octgb_disp_load needs the dispersion-free geometry with a window of ones (plain linearisation)");
        require(n_bscans >= 1 && rep >= 1, "n_bscans and rep must be >= 1");
        require(hann != nullptr, "hann is NULL");
        const int B = n_bscans * rep, nx = interf - apod;
        const size_t lines = static_cast<size_t>(B) * nx;
        // linearised interferogram (window 1: the kernel's output is sum + m)
        // windowed in float64 and rounded once, as (eq * hann).astype(complex64)
        // (dispersion.py:84), written by the spectral kernel itself
        ck(c->disp_x.ensure(lines * kN * sizeof(float)), "cudaMalloc(X)");
        // the window in float64, and split hi + lo in float32 for the kernel's
        // float32 form of the float64 product
        std::vector<double> hw(kN * 2);
        for (int j = 0; j < kN; ++j) {
            const float hi = static_cast<float>(hann[j]);
            reinterpret_cast<float*>(hw.data() + kN)[2 * j] = hi;
            reinterpret_cast<float*>(hw.data() + kN)[2 * j + 1] = static_cast<float>(hann[j] - static_cast<double>(hi));
            hw[j] = hann[j];
        }
        ck(c->disp_hann.ensure(kN * 2 * sizeof(double)), "cudaMalloc(hann)");
        ck(cudaMemcpyAsync(c->disp_hann.p, hw.data(), hw.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream),
           "H2D hann");
        run_spectral(c, raw, dtype, loc, B, interf, apod, kModeLinHann, c->disp_x.as<float>(), 0, 0, nullptr,
                     c->disp_hann.as<double>(), reinterpret_cast<const float2*>(c->disp_hann.as<double>() + kN));
        check_status(c);
        c->disp_b = n_bscans;
        c->disp_rep = rep;
        c->disp_nx = nx;
    });
}

int octgb_disp_lines(octgb_ctx* c, float* out, int out_loc) {
    return guarded(c, [&] {
        require(c->disp_b > 0, "octgb_disp_load has not been called");
        require(out != nullptr, "out is NULL");
        copy_out(c, out, out_loc, c->disp_x.p,
                 static_cast<size_t>(c->disp_b) * c->disp_rep * c->disp_nx * kN * sizeof(float));
        check_status(c);
    });
}

int octgb_disp_set_dk2(octgb_ctx* c, const double* dk2) {
    return guarded(c, [&] {
        require(dk2 != nullptr, "dk2 is NULL");
        c->dk2.assign(dk2, dk2 + kN);
    });
}

namespace {
// exp(-i beta dk^2) in float64, rounded to complex64 (dispersion.py:88-89), times 1/N
void disp_phase_rows(const octgb_ctx* c, const double* betas, int n, float2* ph) {
    for (int gi = 0; gi < n; ++gi) {
        const double beta = betas[gi];
        for (int j = 0; j < kN; ++j) {
            const double t = beta * c->dk2[j];
            ph[static_cast<size_t>(gi) * kN + j] = make_float2(static_cast<float>(std::cos(t)) * (1.0f / kN),
                                                               static_cast<float>(-std::sin(t)) * (1.0f / kN));
        }
    }
}
}  // namespace

int octgb_disp_eval(octgb_ctx* c, int n_beta, const double* betas, int b0, int nb, int metric, int64_t top_k,
                    int z_min, double* scores, float* mag, int mag_loc) {
    return guarded(c, [&] {
        require(c->disp_b > 0, "octgb_disp_load has not been called");
        require(static_cast<int>(c->dk2.size()) == kN, "octgb_disp_set_dk2 has not been called");
        require(n_beta >= 1 && betas != nullptr, "no betas");
        require(b0 >= 0 && nb >= 1 && b0 + nb <= c->disp_b, "B-scan range outside the loaded B-scans");
        require(metric >= 0 && metric <= 4, "metric must be 0 (none) .. 4");
        require(metric == 0 || scores != nullptr, "scores is NULL");
        require(metric != 1 || (top_k >= 1 && top_k <= static_cast<int64_t>(c->disp_nx) * (kHalf - z_min)),
                "top_k out of range");
        require(z_min >= 0 && z_min < kHalf, "z_min must be in [0, N/2)");
        require(metric != 0 || mag != nullptr, "nothing to compute (metric 0 and no magnitude output)");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        const int nx = c->disp_nx;
        const size_t seg_floats = static_cast<size_t>(nx) * kHalf;
        // betas in chunks whose magnitudes fit a 1 GiB scratch (unless written to the caller's device buffer)
        const int per = mag != nullptr && mag_loc == OCTGB_DEVICE
                            ? n_beta
                            : std::max(1, static_cast<int>((size_t(1) << 30) / (seg_floats * nb * sizeof(float))));
        std::vector<float2> ph(static_cast<size_t>(std::min(per, n_beta)) * kN);
        ck(c->disp_score.ensure(static_cast<size_t>(n_beta) * nb * sizeof(double)), "cudaMalloc(scores)");
        for (int g0 = 0; g0 < n_beta; g0 += per) {
            const int ng = std::min(per, n_beta - g0);
            disp_phase_rows(c, betas + g0, ng, ph.data());
            ck(c->disp_phase.ensure(static_cast<size_t>(per) * kN * sizeof(float2)), "cudaMalloc(phase)");
            ck(cudaMemcpyAsync(c->disp_phase.p, ph.data(), static_cast<size_t>(ng) * kN * sizeof(float2),
                               cudaMemcpyHostToDevice, c->stream),
               "H2D phase");
            float* A = nullptr;
            if (mag != nullptr && mag_loc == OCTGB_DEVICE) {
                A = mag + static_cast<size_t>(g0) * nb * seg_floats;
            } else {
                ck(c->disp_a.ensure(static_cast<size_t>(per) * nb * seg_floats * sizeof(float)), "cudaMalloc(A)");
                A = c->disp_a.as<float>();
            }
            DispArgs a{};
            a.X = c->disp_x.as<float>();
            a.phase = c->disp_phase.as<float2>();
            a.tw = c->tw.as<float2>();
            a.A = A;
            a.n_beta = ng;
            a.nb = nb;
            a.b0 = b0;
            a.nx = nx;
            a.rep = c->disp_rep;
            ck(launch_disp_mag(a, c->num_sms, c->stream), "dispersion magnitude kernel");
            c->launches++;
            if (metric != 0) {
                ck(launch_disp_metric(A, ng * nb, nx, z_min, metric, static_cast<unsigned int>(top_k),
                                      c->disp_score.as<double>() + static_cast<size_t>(g0) * nb, c->stream),
                   "dispersion metric kernel");
                c->launches++;
            }
            if (mag != nullptr && mag_loc != OCTGB_DEVICE)
                copy_out(c, mag + static_cast<size_t>(g0) * nb * seg_floats, OCTGB_HOST, A,
                         static_cast<size_t>(ng) * nb * seg_floats * sizeof(float));
        }
        if (metric != 0)
            ck(cudaMemcpyAsync(scores, c->disp_score.p, static_cast<size_t>(n_beta) * nb * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream),
               "D2H scores");
        check_status(c);
    });
}

namespace {
void xprofile(octgb_ctx* c, const float* mag, int mag_loc, int n_frames, int nx, int nz, int ignore_nan,
              int mean_mode, double* out) {
    require(mag != nullptr && out != nullptr, "NULL buffer");
    require(n_frames >= 1 && nx >= 1 && nx <= 4096 && nz >= 1, "shape must have 1..4096 A-scans per frame");
    const size_t n = static_cast<size_t>(n_frames) * nx * nz;
    const float* src = mag;
    if (mag_loc != OCTGB_DEVICE) {
        ck(c->out.ensure(n * sizeof(float)), "cudaMalloc(mag)");
        ck(cudaMemcpyAsync(c->out.p, mag, n * sizeof(float), cudaMemcpyHostToDevice, c->stream), "H2D mag");
        src = c->out.as<float>();
    }
    ck(c->xmed.ensure(static_cast<size_t>(n_frames) * nz * sizeof(double)), "cudaMalloc(median)");
    ck(launch_xmedian(src, n_frames, nx, nz, ignore_nan, mean_mode, c->xmed.as<double>(), c->stream),
       "x-profile kernel");
    c->launches++;
    ck(cudaMemcpyAsync(out, c->xmed.p, static_cast<size_t>(n_frames) * nz * sizeof(double),
                       cudaMemcpyDeviceToHost, c->stream),
       "D2H profile");
    check_status(c);
}
}  // namespace

int octgb_xmedian(octgb_ctx* c, const float* mag, int mag_loc, int n_frames, int nx, int nz, int ignore_nan,
                  double* out) {
    return guarded(c, [&] { xprofile(c, mag, mag_loc, n_frames, nx, nz, ignore_nan, 0, out); });
}

int octgb_xmean(octgb_ctx* c, const float* mag, int mag_loc, int n_frames, int nx, int nz, double* out) {
    return guarded(c, [&] { xprofile(c, mag, mag_loc, n_frames, nx, nz, 1, 1, out); });
}

// ---------------------------------------------------------------------------
// Legacy TIFF encoding (io/tiff_writer.py:53-71).

int octgb_quantise_double(octgb_ctx* c, const float* db, int64_t n, int db_loc, double p1, double p2, double c1,
                          double c2, uint16_t* bits, int bits_loc) {
    return guarded(c, [&] {
        require(db != nullptr && bits != nullptr && n >= 0, "bad quantisation arguments");
        if (p1 > p2) std::swap(p1, p2);
        if (c1 > c2) std::swap(c1, c2);
        require(c2 > c1, "clim must have c1 < c2");
        if (n == 0) return;
        const float* src = db;
        if (db_loc != OCTGB_DEVICE) {
            ck(c->dbbuf.ensure(n * sizeof(float)), "cudaMalloc(db)");
            ck(cudaMemcpyAsync(c->dbbuf.p, db, n * sizeof(float), cudaMemcpyHostToDevice, c->stream), "H2D db");
            src = c->dbbuf.as<float>();
        }
        uint16_t* dst = bits;
        if (bits_loc != OCTGB_DEVICE) {
            ck(c->enc_bits.ensure(n * sizeof(uint16_t)), "cudaMalloc(bits)");
            dst = c->enc_bits.as<uint16_t>();
        }
        ck(c->qtable.ensure(kQuantTable * sizeof(float)), "cudaMalloc(table)");
        // a plane without finite values has NaN plane clim: all its codes are 0
        // either way, so it takes the single quantisation
        const bool twice = std::isfinite(p1) && std::isfinite(p2) && p2 > p1;
        ck(launch_quantise(src, n, twice ? p1 : c1, twice ? p2 : c2, c->qtable.as<float>(), dst, c->stream),
           "quantise kernels");
        c->launches += 2;
        if (twice) {
            ck(c->enc_lut.ensure(65536 * sizeof(uint16_t)), "cudaMalloc(lut)");
            ck(launch_requant(dst, n, p1, p2, c1, c2, c->enc_lut.as<uint16_t>(), c->stream), "re-quantise kernels");
            c->launches += 2;
        }
        if (bits_loc != OCTGB_DEVICE) copy_out(c, bits, OCTGB_HOST, dst, n * sizeof(uint16_t));
        check_status(c);
    });
}

int octgb_packbits(octgb_ctx* c, const uint16_t* img, int img_loc, int rows, int cols, uint8_t* out,
                   int64_t capacity, int* row_sizes, int64_t* total) {
    return guarded(c, [&] {
        require(img && out && row_sizes && total, "NULL buffer");
        require(rows >= 0 && cols >= 1, "bad image shape");
        *total = 0;
        if (rows == 0) return;
        const size_t n = static_cast<size_t>(rows) * cols;
        const uint16_t* src = img;
        if (img_loc != OCTGB_DEVICE) {
            ck(c->enc_bits.ensure(n * sizeof(uint16_t)), "cudaMalloc(image)");
            ck(cudaMemcpyAsync(c->enc_bits.p, img, n * sizeof(uint16_t), cudaMemcpyHostToDevice, c->stream),
               "H2D image");
            src = c->enc_bits.as<uint16_t>();
        }
        const int slot = packbits_slot(cols);
        ck(c->enc_slots.ensure(static_cast<size_t>(rows) * slot), "cudaMalloc(slots)");
        ck(c->enc_sizes.ensure(static_cast<size_t>(rows) * sizeof(int)), "cudaMalloc(sizes)");
        ck(launch_packbits(src, rows, cols, c->enc_slots.as<uint8_t>(), c->enc_sizes.as<int>(), c->stream),
           "packbits kernel");
        c->launches++;
        std::vector<uint8_t> h(static_cast<size_t>(rows) * slot);
        ck(cudaMemcpyAsync(row_sizes, c->enc_sizes.p, static_cast<size_t>(rows) * sizeof(int), cudaMemcpyDeviceToHost,
                           c->stream),
           "D2H sizes");
        ck(cudaMemcpyAsync(h.data(), c->enc_slots.p, h.size(), cudaMemcpyDeviceToHost, c->stream), "D2H slots");
        check_status(c);
        int64_t off = 0;
        for (int r = 0; r < rows; ++r) off += row_sizes[r];
        require(off <= capacity, "output capacity too small for the packed image");
        off = 0;
        for (int r = 0; r < rows; ++r) {
            memcpy(out + off, h.data() + static_cast<size_t>(r) * slot, row_sizes[r]);
            off += row_sizes[r];
        }
        *total = off;
    });
}

// ---------------------------------------------------------------------------
// Rare raw formats (core/spectral.py:20-82,168-177; pipeline.py:274-285).

int octgb_prepare_raw(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int n_lines, int apod, int binning,
                      int apod_mode, int apod_group, float* out, int out_loc, int* out_lines) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, n_lines, apod_mode == 1 ? 1 : apod);
        require(out != nullptr && out_lines != nullptr, "NULL output");
        PrepArgs a{};
        prep_args(a, raw, B, n_lines, apod, binning, apod_mode, apod_group);
        *out_lines = a.a_out + a.n_kept;
        if (B == 0) return;
        run_prepare(c, a, dtype, loc);
        copy_out(c, out, out_loc, c->prep.p, static_cast<size_t>(B) * (a.a_out + a.n_kept) * kN * sizeof(float));
        check_status(c);
    });
}

int octgb_srr_decode(octgb_ctx* c, const uint16_t* words, int loc, int n_files, int file_lines, int n, int apod_start,
                     int apod_end, int scan_start, int scan_end, int16_t* out, int out_loc) {
    return guarded(c, [&] {
        require(words != nullptr && out != nullptr, "NULL buffer");
        require(n_files >= 0 && file_lines >= 1 && n >= 1, "bad SRR file shape");
        require(apod_start >= 0 && apod_start < apod_end && apod_end <= file_lines,
                "apodisation lines must be a non-empty range inside the file");
        require(scan_start >= 0 && scan_start < scan_end && scan_end <= file_lines,
                "scan lines must be a non-empty range inside the file");
        const int na = apod_end - apod_start, lines_out = na + (scan_end - scan_start);
        if (n_files == 0) return;
        const size_t out_bytes = static_cast<size_t>(n_files) * lines_out * n * sizeof(int16_t);
        int16_t* dst = out;
        if (out_loc != OCTGB_DEVICE) {
            ck(c->srr.ensure(out_bytes), "cudaMalloc(srr)");
            dst = c->srr.as<int16_t>();
        }
        if (loc == OCTGB_DEVICE) {
            ck(launch_srr_decode(words, static_cast<int64_t>(file_lines) * n, apod_start, na, scan_start, lines_out, n,
                                 n_files, dst, c->stream),
               "SRR decode kernel");
        } else {
            // only the used lines cross the link: two strided copies into the
            // output layout, then the 12-bit decode in place
            const size_t row = static_cast<size_t>(n) * sizeof(uint16_t);
            const size_t sp = static_cast<size_t>(file_lines) * row, dp = static_cast<size_t>(lines_out) * row;
            ck(cudaMemcpy2DAsync(dst, dp, words + static_cast<size_t>(apod_start) * n, sp, na * row, n_files,
                                 cudaMemcpyHostToDevice, c->stream),
               "H2D SRR apodisation lines");
            ck(cudaMemcpy2DAsync(dst + static_cast<size_t>(na) * n, dp, words + static_cast<size_t>(scan_start) * n, sp,
                                 (scan_end - scan_start) * row, n_files, cudaMemcpyHostToDevice, c->stream),
               "H2D SRR scan lines");
            ck(launch_srr_decode(reinterpret_cast<const uint16_t*>(dst), static_cast<int64_t>(lines_out) * n, 0, na, na,
                                 lines_out, n, n_files, dst, c->stream),
               "SRR decode kernel");
        }
        c->launches++;
        if (out_loc != OCTGB_DEVICE) copy_out(c, out, OCTGB_HOST, dst, out_bytes);
        check_status(c);
    });
}

int octgb_average_repeats(octgb_ctx* c, const float* mag, int mag_loc, int n_frames, int bscan_avg, int size_x,
                          int ascan_avg, int nz, float* out, int out_loc) {
    return guarded(c, [&] {
        require(mag && out, "NULL buffer");
        require(n_frames >= 0 && bscan_avg >= 1 && ascan_avg >= 1 && size_x >= 1 && nz >= 1, "bad repeat shape");
        if (n_frames == 0) return;
        const size_t in_n = static_cast<size_t>(n_frames) * bscan_avg * size_x * ascan_avg * nz;
        const size_t out_n = static_cast<size_t>(n_frames) * size_x * nz;
        const float* src = mag;
        if (mag_loc != OCTGB_DEVICE) {
            ck(c->magrep.ensure(in_n * sizeof(float)), "cudaMalloc(mag)");
            ck(cudaMemcpyAsync(c->magrep.p, mag, in_n * sizeof(float), cudaMemcpyHostToDevice, c->stream), "H2D mag");
            src = c->magrep.as<float>();
        }
        float* dst = out;
        if (out_loc != OCTGB_DEVICE) {
            ck(c->magbuf.ensure(out_n * sizeof(float)), "cudaMalloc(out)");
            dst = c->magbuf.as<float>();
        }
        ck(launch_avg_repeats(src, n_frames, bscan_avg, size_x, ascan_avg, nz, dst, c->stream), "repeat kernel");
        c->launches++;
        if (out_loc != OCTGB_DEVICE) copy_out(c, out, OCTGB_HOST, dst, out_n * sizeof(float));
        check_status(c);
    });
}

int octgb_row_add_batch_ex(octgb_ctx* c, int plan_id, const void* raw, int dtype, int loc, int n_files, int n_lines,
                           int apod, int binning, int apod_mode, int bscan_avg, int ascan_avg, const int64_t* frame_idx,
                           int n_frames, int frame_offset) {
    return guarded(c, [&] {
        if (!c->row_open) throw Error(OCTGB_ERR_STATE, "octgb_row_begin has not been called");
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        require(plan_id >= 0 && plan_id < static_cast<int>(c->plans.size()), "bad plan id");
        const Plan& p = *c->plans[plan_id];
        validate_raw(raw, dtype, loc, n_files, n_lines, apod_mode == 1 ? 1 : apod);
        require(bscan_avg >= 1 && ascan_avg >= 1, "repeat counts must be >= 1");
        require(n_files == n_frames * bscan_avg, "n_files must be n_frames x bscan_avg (repeats consecutive)");
        require(frame_offset >= 0 && frame_offset + n_frames <= c->row_nf, "frames outside the row");
        require(frame_idx != nullptr, "frame_idx is NULL");
        PrepArgs a{};
        const bool prep = prep_args(a, raw, n_files, n_lines, apod, binning, apod_mode, bscan_avg);
        require(a.n_kept % ascan_avg == 0, "A-lines are not a whole number of A-scan repeats");
        const int size_x = a.n_kept / ascan_avg;
        require(size_x == p.n_tile_x, "A-scans per B-scan differ from the plan's tile width");
        require(p.n_out_z == c->row_nz && p.c0 + p.C <= c->row_nx, "plan does not fit the row");
        std::vector<int> fy(n_frames > 0 ? n_frames : 1);
        bool contiguous = true;
        for (int f = 0; f < n_frames; ++f) {
            require(!p.opc || (frame_idx[f] >= 0 && frame_idx[f] < p.n_y), "frame index outside the scan");
            fy[f] = static_cast<int>(frame_idx[f]);
            contiguous = contiguous && frame_idx[f] == frame_idx[0] + f;
        }
        if (n_frames == 0) return;
        // spectral input: the prepared float32 batch, or the raw batch itself
        const void* src = raw;
        int sdt = dtype, sloc = loc, s_lines = n_lines, s_apod = apod;
        if (prep) {
            run_prepare(c, a, dtype, loc);
            src = c->prep.p;
            sdt = OCTGB_F32;
            sloc = OCTGB_DEVICE;
            s_lines = a.a_out + a.n_kept;
            s_apod = a.a_out;
        }
        const bool rep = bscan_avg > 1 || ascan_avg > 1;
        ck(c->magbuf.ensure(static_cast<size_t>(n_frames) * size_x * kHalf * sizeof(float)), "cudaMalloc(mag)");
        float* m = c->magbuf.as<float>();
        if (rep) {
            ck(c->magrep.ensure(static_cast<size_t>(n_files) * a.n_kept * kHalf * sizeof(float)), "cudaMalloc(mag)");
            m = c->magrep.as<float>();
        }
        run_spectral(c, src, sdt, sloc, n_files, s_lines, s_apod, kModeMag, m, 0, 0, nullptr);
        if (rep) {
            ck(launch_avg_repeats(m, n_frames, bscan_avg, size_x, ascan_avg, kHalf, c->magbuf.as<float>(), c->stream),
               "repeat kernel");
            c->launches++;
        }
        stitch_row(c, p, c->magbuf.as<float>(), fy, contiguous, n_frames, frame_offset);
    });
}

// ---------------------------------------------------------------------------
// Precision form: the sinc on the tensor cores (split-FP16, three products).

namespace {
// X (B * nx lines of kN float32, device) = linearised interferogram of a raw batch
float* precision_linearise(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod,
                           float* x_dev = nullptr) {
    if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
    if (!c->prec_ok)
        throw Error(OCTGB_ERR_STATE, "the precision form needs every 64-output block's sinc band within 96 samples");
    if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
    const int nx = interf - apod;
    const int64_t n = static_cast<int64_t>(B) * nx;
    const size_t bytes = static_cast<size_t>(B) * interf * kN * raw_elem(dtype);
    const void* rd = stage_raw(c, raw, dtype, loc, bytes);
    // (+ one window of padding: the sinc kernel copies whole 96-sample windows of the sums)
    ck(c->apod.ensure(static_cast<size_t>(B) * kN * sizeof(double) + kPKW * sizeof(int) + 16), "cudaMalloc(apod)");
    SpectralArgs a{};
    a.raw = rd;
    a.seg[0] = rd;
    a.n_seg = 1;
    a.B = B;
    a.interf = interf;
    a.apod = apod;
    a.nx = nx;
    a.n_ascans = n;
    float* X = x_dev;
    if (X == nullptr) {
        ck(c->prec_x.ensure(static_cast<size_t>(n) * kN * sizeof(float)), "cudaMalloc(X)");
        X = c->prec_x.as<float>();
    }
    ck(c->prec_m.ensure(static_cast<size_t>(n) * sizeof(float)), "cudaMalloc(line means)");
    if (dtype != OCTGB_F32) {
        // integer raws: the sinc kernel reads the raw window itself (no d' in memory)
        ck(c->prec_hi.ensure(static_cast<size_t>(n) * sizeof(long long)), "cudaMalloc(line sums)");
        CUtensorMap mr;
        if (!encode_raw_map(&mr, rd, B, interf, apod)) throw Error(OCTGB_ERR_CUDA, "cuTensorMapEncodeTiled failed");
        ck(launch_prec_sinc_raw(a, dtype, mr, c->prec_w.as<uint8_t>(), c->prec_kb.as<int>(), c->apod.as<int>(),
                                c->prec_hi.as<long long>(), c->prec_m.as<float>(), X, c->status_dev, c->num_sms,
                                c->stream),
           "tensor-core sinc kernels");
        c->launches += 3;
        return X;
    }
    ck(c->prec_hi.ensure(static_cast<size_t>(n) * kN * sizeof(__half)), "cudaMalloc(d hi)");
    ck(c->prec_lo.ensure(static_cast<size_t>(n) * kN * sizeof(__half)), "cudaMalloc(d lo)");
    ck(launch_prec_split(a, dtype, c->apod.p, c->prec_hi.as<__half>(), c->prec_lo.as<__half>(),
                         c->prec_m.as<float>(), c->num_sms, c->stream),
       "background / split kernels");
    CUtensorMap mh, ml;
    if (!encode_prec_map(&mh, c->prec_hi.p, n) || !encode_prec_map(&ml, c->prec_lo.p, n))
        throw Error(OCTGB_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    ck(launch_prec_sinc(mh, ml, c->prec_w.as<uint8_t>(), c->prec_kb.as<int>(), c->prec_m.as<float>(), X, n,
                        c->status_dev, c->num_sms, c->stream),
       "tensor-core sinc kernel");
    c->launches += 3;
    return X;
}
}  // namespace

int octgb_selftest_wait_expiry(octgb_ctx* c, int which, int wait_limit_us) {
    return guarded(c, [&] {
        require(which == 0 || which == 1, "which must be 0 (spectral kernel) or 1 (precision form)");
        require(wait_limit_us >= 100 && wait_limit_us <= 2000000, "wait_limit_us must be in [100, 2000000]");
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (which == 1) require(c->prec_ok, "the geometry has no precision-form (tensor-core) tiles");
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "self-test during graph capture");
        auto set = which == 0 ? set_wait_test_spectral : set_wait_test_precision;
        constexpr unsigned long long kDefaultLimit = 2000000000ull;
        // zero raws, 2 B-scans x (1 apodisation + 256) lines, already on the device
        const int B = 2, interf = 257, apod = 1;
        const size_t bytes = static_cast<size_t>(B) * interf * kN * sizeof(uint16_t);
        ck(c->raw.ensure(bytes), "cudaMalloc(raw)");
        ck(cudaMemsetAsync(c->raw.p, 0, bytes, c->stream), "memset raw");
        ck(set(static_cast<unsigned long long>(wait_limit_us) * 1000ull, 1, c->stream), "set wait limit");
        try {
            if (which == 0) {
                ck(c->magbuf.ensure(static_cast<size_t>(B) * (interf - apod) * kHalf * sizeof(float)),
                   "cudaMalloc(mag)");
                run_spectral(c, c->raw.p, OCTGB_U16, OCTGB_DEVICE, B, interf, apod, kModeMag, c->magbuf.as<float>(), 0,
                             0, nullptr);
            } else {
                precision_linearise(c, c->raw.p, OCTGB_U16, OCTGB_DEVICE, B, interf, apod);
            }
            check_status(c);                    // a wait that expired throws OCTGB_ERR_TIMEOUT here
        } catch (...) {
            set(kDefaultLimit, 0, c->stream);
            throw;
        }
        ck(set(kDefaultLimit, 0, c->stream), "restore wait limit");
        throw Error(OCTGB_ERR_STATE, "self-test: the starved row-copy wait did not expire");
    });
}

int octgb_linearise_precision(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod,
                              float* x, int x_loc) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(x != nullptr, "x is NULL");
        if (B == 0) return;
        if (x_loc == OCTGB_DEVICE) {
            require((reinterpret_cast<uintptr_t>(x) & 15u) == 0, "device x must be 16-byte aligned");
            precision_linearise(c, raw, dtype, loc, B, interf, apod, x);
            if (loc != OCTGB_DEVICE) check_status(c);
            return;
        }
        const float* X = precision_linearise(c, raw, dtype, loc, B, interf, apod);
        copy_out(c, x, x_loc, X, static_cast<size_t>(B) * (interf - apod) * kN * sizeof(float));
        check_status(c);
    });
}

int octgb_magnitude_exact(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod, float* mag,
                          int mag_loc) {
    return guarded(c, [&] {
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(dtype == OCTGB_U16 || dtype == OCTGB_I16,
                "the float64 form takes integer raws (its background is formed exactly from integer sums)");
        require(mag != nullptr, "mag is NULL");
        if (B == 0) return;
        const size_t bytes = static_cast<size_t>(B) * interf * kN * raw_elem(dtype);
        const void* rd = stage_raw(c, raw, dtype, loc, bytes);
        const int nx = interf - apod;
        const size_t ob = static_cast<size_t>(B) * nx * kHalf * sizeof(float);
        float* dst = mag;
        if (mag_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(ob), "cudaMalloc(out)");
            dst = c->out.as<float>();
        }
        ck(c->apod.ensure(static_cast<size_t>(B) * kN * sizeof(int)), "cudaMalloc(apodisation sums)");
        ExactArgs a{};
        a.raw = rd;
        a.B = B;
        a.interf = interf;
        a.apod = apod;
        a.nx = nx;
        a.n_ascans = static_cast<int64_t>(B) * nx;
        a.start = c->start.as<int>();
        a.w = c->ex_w.as<double>();
        a.taps = c->taps;
        a.win = c->ex_win.as<double2>();
        a.tw = c->ex_tw.as<double2>();
        a.mag = dst;
        ck(launch_exact(a, dtype, c->apod.as<int>(), c->num_sms, c->stream), "float64 spectral kernels");
        c->launches += 2;
        if (mag_loc != OCTGB_DEVICE) copy_out(c, mag, OCTGB_HOST, dst, ob);
        if (mag_loc != OCTGB_DEVICE || loc != OCTGB_DEVICE) check_status(c);
    });
}

int octgb_magnitude_precision(octgb_ctx* c, const void* raw, int dtype, int loc, int B, int interf, int apod,
                              float* mag, int mag_loc) {
    return guarded(c, [&] {
        validate_raw(raw, dtype, loc, B, interf, apod);
        require(mag != nullptr, "mag is NULL");
        if (B == 0) return;
        const float* X = precision_linearise(c, raw, dtype, loc, B, interf, apod);
        const size_t ob = static_cast<size_t>(B) * (interf - apod) * kHalf * sizeof(float);
        float* dst = mag;
        if (mag_loc != OCTGB_DEVICE) {
            ck(c->out.ensure(ob), "cudaMalloc(out)");
            dst = c->out.as<float>();
        }
        // window (Hann/rms x dispersion phase / N), inverse FFT, |.|: the scorer's FFT kernel
        DispArgs a{};
        a.X = X;
        a.phase = c->win.as<float2>();
        a.tw = c->tw.as<float2>();
        a.A = dst;
        a.n_beta = 1;
        a.nb = B;
        a.b0 = 0;
        a.nx = interf - apod;
        a.rep = 1;
        ck(launch_disp_mag(a, c->num_sms, c->stream), "FFT kernel");
        c->launches++;
        if (mag_loc != OCTGB_DEVICE) copy_out(c, mag, OCTGB_HOST, dst, ob);
        if (mag_loc != OCTGB_DEVICE || loc != OCTGB_DEVICE) check_status(c);
    });
}

// ---------------------------------------------------------------------------
// Learned beta/focus estimator: device pointers only, asynchronous on the
// context's stream (no counterpart in the reference).

int octgb_disp_images(octgb_ctx* c, int n_beta, const double* betas, int b0, int nb, int z_keep, float* img,
                      int normalise) {
    return guarded(c, [&] {
        require(c->disp_b > 0, "octgb_disp_load has not been called");
        require(static_cast<int>(c->dk2.size()) == kN, "octgb_disp_set_dk2 has not been called");
        require(n_beta >= 1 && betas != nullptr, "no betas");
        require(b0 >= 0 && nb >= 1 && b0 + nb <= c->disp_b, "B-scan range outside the loaded B-scans");
        require(z_keep >= 1 && z_keep <= kHalf, "z_keep must be in [1, N/2]");
        require(img != nullptr, "img is NULL");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        const int nx = c->disp_nx;
        std::vector<float2> ph(static_cast<size_t>(n_beta) * kN);
        disp_phase_rows(c, betas, n_beta, ph.data());
        ck(c->disp_phase.ensure(ph.size() * sizeof(float2)), "cudaMalloc(phase)");
        ck(cudaMemcpyAsync(c->disp_phase.p, ph.data(), ph.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream),
           "H2D phase");
        const size_t cols = static_cast<size_t>(n_beta) * nb * nx * 256;
        ck(c->disp_a.ensure(cols * sizeof(float)), "cudaMalloc(columns)");
        DispArgs a{};
        a.X = c->disp_x.as<float>();
        a.phase = c->disp_phase.as<float2>();
        a.tw = c->tw.as<float2>();
        a.A = nullptr;
        a.zcol = c->disp_a.as<float>();
        a.z_keep = z_keep;
        a.n_beta = n_beta;
        a.nb = nb;
        a.b0 = b0;
        a.nx = nx;
        a.rep = c->disp_rep;
        ck(launch_disp_mag(a, c->num_sms, c->stream), "dispersion magnitude kernel");
        ck(launch_image_cols(a.zcol, n_beta, nb, nx, z_keep, img, c->stream), "image column kernel");
        c->launches += 2;
        if (normalise) {
            ck(launch_image_norm(img, nb, static_cast<int64_t>(n_beta) * 256 * 256, c->stream), "image norm kernel");
            c->launches++;
        }
    });
}

int octgb_cnn_images(octgb_ctx* c, const float* mag, int n_probe, int nb, int nx, int z_keep, float* img,
                     int normalise) {
    return guarded(c, [&] {
        require(mag && img, "NULL buffer");
        require(n_probe >= 1 && nb >= 1 && nx >= 1 && z_keep >= 1 && z_keep <= kHalf, "bad image shape");
        ck(launch_image_pool(mag, n_probe, nb, nx, z_keep, img, c->stream), "image pool kernel");
        c->launches++;
        if (normalise) {
            ck(launch_image_norm(img, nb, static_cast<int64_t>(n_probe) * 256 * 256, c->stream), "image norm kernel");
            c->launches++;
        }
    });
}

int octgb_cnn_conv3x3(octgb_ctx* c, const float* x, const float* w, const float* b, float* y, int n, int cin,
                      int cout, int h, int wd) {
    return guarded(c, [&] {
        require(x && w && y, "NULL buffer");
        require(n >= 1 && cin >= 1 && cout >= 1 && h >= 1 && wd >= 1 && n <= 65535, "bad convolution shape");
        ck(launch_conv3x3(x, w, b, y, n, cin, cout, h, wd, c->stream), "conv kernel");
        c->launches++;
    });
}

int octgb_cnn_conv3x3_tc(octgb_ctx* c, const float* x, const float* w, const float* b, float* y, int n, int cin,
                         int cout, int h, int wd) {
    return guarded(c, [&] {
        require(x && w && y, "NULL buffer");
        require(n >= 1 && h >= 1 && wd >= 1, "bad convolution shape");
        require(conv3x3_tc_supported(cin, cout, h, wd),
                "tensor-core convolution: 1 <= cin <= 32, cout a multiple of 32 up to 128, and the width a "
                "multiple of 128 or a divisor of 128 whose row count divides the height");
        ck(launch_conv3x3_tc(x, w, b, y, n, cin, cout, h, wd, 0, c->status_dev, c->stream), "tensor-core conv kernel");
        c->launches++;
    });
}

int octgb_cnn_conv3x3_relu_pool_tc(octgb_ctx* c, const float* x, const float* w, const float* b, float* p, int n,
                                   int cin, int cout, int h, int wd) {
    return guarded(c, [&] {
        require(x && w && p, "NULL buffer");
        require(n >= 1 && h >= 1 && wd >= 1, "bad convolution shape");
        require(conv3x3_tc_pool_supported(cin, cout, h, wd),
                "fused tensor-core convolution + pool: 1 <= cin <= 32, cout a multiple of 32 up to 128, the width "
                "a multiple of 128 and the height even");
        ck(launch_conv3x3_tc(x, w, b, p, n, cin, cout, h, wd, 1, c->status_dev, c->stream),
           "tensor-core conv + pool kernel");
        c->launches++;
    });
}

int octgb_cnn_conv3x3_bwd(octgb_ctx* c, const float* x, const float* w, const float* dy, float* dx, float* dw,
                          float* db, float* w_scratch, int n, int cin, int cout, int h, int wd) {
    return guarded(c, [&] {
        require(x && w && dy && dw && db, "NULL buffer");
        require(n >= 1 && cin >= 1 && cout >= 1 && h >= 1 && wd >= 1 && n <= 65535, "bad convolution shape");
        ck(launch_conv3x3_wgrad(x, dy, dw, n, cin, cout, h, wd, c->stream), "conv weight-gradient kernel");
        ck(c->bias_part.ensure(static_cast<size_t>(n) * cout * sizeof(float)), "cudaMalloc(bias partial sums)");
        ck(launch_bias_grad(dy, n, cout, static_cast<int64_t>(h) * wd, db, c->bias_part.as<float>(), c->stream),
           "bias-gradient kernel");
        c->launches += (static_cast<int64_t>(h) * wd) % 4 == 0 ? 3 : 2;
        if (dx != nullptr) {
            require(w_scratch != nullptr, "w_scratch is NULL");
            ck(launch_flip_weights(w, cout, cin, w_scratch, c->stream), "weight flip kernel");
            ck(launch_conv3x3(dy, w_scratch, nullptr, dx, n, cout, cin, h, wd, c->stream), "conv kernel");
            c->launches += 2;
        }
    });
}

int octgb_cnn_conv3x3_bwd_tc(octgb_ctx* c, const float* x, const float* w, const float* dy, float* dx, float* dw,
                             float* db, float* w_scratch, int n, int cin, int cout, int h, int wd) {
    return guarded(c, [&] {
        require(x && w && dy && dw && db, "NULL buffer");
        require(n >= 1 && cin >= 1 && cout >= 1 && h >= 1 && wd >= 1, "bad convolution shape");
        const size_t parts = conv3x3_wgrad_tc_partials(n, cin, cout, h, wd, c->num_sms);
        require(parts > 0, "tensor-core weight gradient: 1 <= cin <= 48, 1 <= cout <= 128 and a band of rows "
                           "dividing the height whose staged input fits in shared memory");
        ck(c->wgrad_part.ensure(parts * sizeof(float)), "cudaMalloc(weight-gradient partial sums)");
        ck(launch_conv3x3_wgrad_tc(x, dy, dw, n, cin, cout, h, wd, c->wgrad_part.as<float>(), c->num_sms,
                                   c->status_dev, c->stream),
           "tensor-core weight-gradient kernel");
        ck(c->bias_part.ensure(static_cast<size_t>(n) * cout * sizeof(float)), "cudaMalloc(bias partial sums)");
        ck(launch_bias_grad(dy, n, cout, static_cast<int64_t>(h) * wd, db, c->bias_part.as<float>(), c->stream),
           "bias-gradient kernel");
        c->launches += 2 + ((static_cast<int64_t>(h) * wd) % 4 == 0 ? 2 : 1);
        if (dx != nullptr) {
            require(w_scratch != nullptr, "w_scratch is NULL");
            ck(launch_flip_weights(w, cout, cin, w_scratch, c->stream), "weight flip kernel");
            // the data gradient is the convolution of dy with the flipped kernel
            // (cout -> cin channels): BF16 tensor cores where the shape allows
            if (conv3x3_tc_supported(cout, cin, h, wd))
                ck(launch_conv3x3_tc(dy, w_scratch, nullptr, dx, n, cout, cin, h, wd, 0, c->status_dev, c->stream,
                                     true),
                   "tensor-core conv kernel");
            else
                ck(launch_conv3x3(dy, w_scratch, nullptr, dx, n, cout, cin, h, wd, c->stream), "conv kernel");
            c->launches += 2;
        }
    });
}

int octgb_cnn_relu_pool(octgb_ctx* c, const float* y, float* p, int64_t planes, int h, int wd) {
    return guarded(c, [&] {
        require(y && p && planes >= 1 && h >= 2 && wd >= 2 && h % 2 == 0 && wd % 2 == 0, "bad pooling shape");
        ck(launch_relu_pool(y, planes, h, wd, p, c->stream), "relu/pool kernel");
        c->launches++;
    });
}

int octgb_cnn_relu_pool_bwd(octgb_ctx* c, const float* dp, const float* y, float* dy, int64_t planes, int h, int wd) {
    return guarded(c, [&] {
        require(dp && y && dy && planes >= 1 && h % 2 == 0 && wd % 2 == 0, "bad pooling shape");
        ck(launch_relu_pool_bwd(dp, y, planes, h, wd, dy, c->stream), "relu/pool gradient kernel");
        c->launches++;
    });
}

int octgb_cnn_dense(octgb_ctx* c, const float* x, const float* w, const float* b, float* pre, float* act, int m,
                    int in, int out) {
    return guarded(c, [&] {
        require(x && w && b && pre && m >= 1 && in >= 1 && out >= 1, "bad dense shape");
        // few output tiles over a long K (the flattened features): split K across the SMs
        const int S = gemm_splits(m, out, in, c->num_sms);
        if (S > 1) ck(c->gemm_part.ensure(static_cast<size_t>(S) * m * out * sizeof(float)), "cudaMalloc(gemm)");
        ck(launch_gemm_split(x, in, 1, w, 1, in, pre, out, m, out, in, 0, S, c->gemm_part.as<float>(), c->stream),
           "gemm kernel");
        ck(launch_bias_relu(pre, b, m, out, act, c->stream), "bias kernel");
        c->launches += S > 1 ? 3 : 2;
    });
}

int octgb_cnn_dense_bwd(octgb_ctx* c, const float* x, const float* w, float* dy, const float* pre, float* dx,
                        float* dw, float* db, int m, int in, int out) {
    return guarded(c, [&] {
        require(x && w && dy && dw && db && m >= 1 && in >= 1 && out >= 1, "bad dense shape");
        if (pre != nullptr) {
            ck(launch_relu_bwd(dy, pre, static_cast<int64_t>(m) * out, c->stream), "relu gradient kernel");
            c->launches++;
        }
        ck(launch_gemm(dy, 1, out, x, in, 1, dw, in, out, in, m, 0, c->stream), "gemm kernel");
        ck(launch_bias_grad(dy, m, out, 1, db, nullptr, c->stream), "bias-gradient kernel");
        c->launches += 2;
        if (dx != nullptr) {
            ck(launch_gemm(dy, out, 1, w, in, 1, dx, in, m, in, out, 0, c->stream), "gemm kernel");
            c->launches++;
        }
    });
}

int octgb_cnn_mse(octgb_ctx* c, const float* pred, const float* target, int n, float* grad, double* loss) {
    return guarded(c, [&] {
        require(pred && target && grad && loss && n >= 1, "bad loss arguments");
        ck(launch_mse(pred, target, n, grad, loss, c->stream), "loss kernel");
        c->launches++;
    });
}

int octgb_cnn_adam(octgb_ctx* c, float* p, const float* g, float* m, float* v, int64_t n, float lr, float beta1,
                   float beta2, float eps, int step) {
    return guarded(c, [&] {
        require(p && g && m && v && n >= 1 && step >= 1, "bad optimiser arguments");
        const float c1 = 1.0f - std::pow(beta1, static_cast<float>(step));
        const float c2 = 1.0f - std::pow(beta2, static_cast<float>(step));
        ck(launch_adam(p, g, m, v, n, lr, beta1, beta2, eps, c1, c2, c->stream), "adam kernel");
        c->launches++;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free magnitude entry point.
//
// Some callers cannot call cudaMalloc at the point where they reconstruct:
// an acquisition loop that runs inside a frame-grabber callback (cudaMalloc
// can synchronise the device and stall the camera stream), or a host process
// whose GPU memory is owned by another framework's pooling allocator under a
// fixed budget.  For them octgb_magnitude_noalloc does the work of
// octgb_magnitude on device buffers the caller already owns, and keeps its one
// piece of scratch (the per-B-scan apodisation mean) in the fixed array below
// instead of a context buffer.  The array is part of the loaded library image:
// every GPU that loads the library holds it until the process exits.
namespace {

constexpr int kNoAllocMaxBscans = 64;   // B-scans per call: 64 x 2048 floats = 512 KiB

static __device__ __align__(256) float g_noalloc_apod[kNoAllocMaxBscans * kN];

// Device address of g_noalloc_apod per device: the name is a host-side
// stand-in in host code, so the address is looked up once per device, with
// that device current, and passed to the kernels.
constexpr int kMaxDevices = 64;
std::atomic<float*> g_noalloc_ptr[kMaxDevices];

float* noalloc_scratch(int device) {
    require(device >= 0 && device < kMaxDevices, "device ordinal out of range for the allocation-free path");
    float* p = g_noalloc_ptr[device].load();
    if (p == nullptr) {
        void* addr = nullptr;
        ck(cudaGetSymbolAddress(&addr, g_noalloc_apod), "cudaGetSymbolAddress(allocation-free scratch)");
        p = static_cast<float*>(addr);
        g_noalloc_ptr[device].store(p);
    }
    return p;
}

}  // namespace

extern "C" int octgb_magnitude_noalloc(octgb_ctx* c, const void* raw, int dtype, int B, int interf, int apod,
                                       float* mag) {
    return guarded(c, [&] {
        if (!c->has_geom) throw Error(OCTGB_ERR_STATE, "octgb_set_geometry has not been called");
        if (c->capturing) throw Error(OCTGB_ERR_STATE, "not available during graph capture through this context");
        if (c->cancel.load()) throw Error(OCTGB_ERR_CANCELLED, "cancelled");
        validate_raw(raw, dtype, OCTGB_DEVICE, B, interf, apod);
        require(mag != nullptr, "mag is NULL");
        if (B > kNoAllocMaxBscans)
            throw Error(OCTGB_ERR_ARG, "octgb_magnitude_noalloc: B = " + std::to_string(B) +
                                           " exceeds the allocation-free limit of " +
                                           std::to_string(kNoAllocMaxBscans) + " B-scans per call");
        if (B == 0) return;
        float* scratch = noalloc_scratch(c->device);
        // the same launches as octgb_magnitude, with the apodisation mean in
        // the fixed array; k_apod_mean writes every element the spectral
        // kernel then reads, so nothing in the array needs clearing
        SpectralArgs a{};
        a.raw = raw;
        a.seg[0] = raw;
        a.n_seg = 1;
        a.B = B;
        a.interf = interf;
        a.apod = apod;
        a.nx = interf - apod;
        a.n_ascans = static_cast<int64_t>(B) * (interf - apod);
        a.apod_mean = scratch;
        a.g.w = c->w.as<float>();
        a.g.start = c->start.as<int>();
        a.g.taps = c->taps;
        a.g.win = c->win.as<float2>();
        a.g.tw = c->tw.as<float2>();
        a.g.wsh = c->wsh.as<float>();
        a.g.s0 = c->s0.as<int>();
        a.g.U = c->U;
        a.out = mag;
        a.status = c->status_dev;
        ck(launch_apod_mean(a, dtype, c->stream), "apod kernel");
        c->launches++;
        const int64_t quads = (a.n_ascans + kPerCta - 1) / kPerCta;
        int64_t grid = static_cast<int64_t>(c->num_sms) * spectral_max_ctas_per_sm(dtype, kModeMag);
        if (grid > quads) grid = quads;
        ck(launch_spectral(a, dtype, kModeMag, static_cast<int>(grid), c->stream), "spectral kernel");
        c->launches++;
    });
}
