// multi.cu -- batches whose patterns use different ROI layouts: per pattern a
// set of ROI positions, one ROI size and one fit size.  Every layout's
// reference spectra are computed once (as gpu_offset::allocate_memory does,
// src/gpu_offset.hpp:185-210) and kept resident, grouped by transform size.
// A run launches one persistent fused kernel per transform size over a work
// list of (pattern, ROI, output slot, fit size); sizes without a fused kernel
// run the staged pipeline per pattern.  Runs can be captured in a CUDA graph
// and replayed, and the persistent grid of each size is chosen by timing.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "handle.cuh"

using namespace emida_gb;
using namespace emida_gb::host;

struct emida_gb_multi {
    struct layout {
        uint32_t n_rois = 0, side = 0, roi_base = 0;
        int fitsize = 3, cls = -1;
        emida_gb_handle *h = nullptr;  // reference spectra; staged runs when not fused
    };
    struct size_class {
        uint32_t n = 0;     // fused transform length (>= 2 * side)
        uint32_t side = 0;  // ROI side of every layout in the class
        bool fused = false;
        std::vector<uint2> begins;
        uint2 *d_begins = nullptr;
        size_t begins_cap = 0;
        void *d_spec = nullptr;  // [rois][n/2 + 1][n] complex, column-major per ROI
        size_t spec_cap = 0;     // in ROIs
        const void *hann = nullptr, *twiddles = nullptr;  // owned by the class's first layout
        int grid = 0;  // 0: one wave of resident CTAs (less `reserve`)
        uint32_t ppc = 0;  // ROI pairs per CTA (0: the kernel's default)
    };
    // CTA slots a default (one-wave) launch leaves free for kernels that run
    // beside it, such as the request loop's SM copies of the next rows
    int reserve = 0;
    // Work lists of a run, per size class.  Plain runs rotate through RING
    // sets, so uploading one run's lists waits only for the run RING back, not
    // for the stream; the last set belongs to the captured graph.
    struct work_set {
        std::vector<uint4 *> d_items;  // per size class
        std::vector<size_t> cap;       // bytes
        uint4 *h_stage = nullptr;      // pinned staging of every class's items (and pointers)
        size_t h_cap = 0;              // bytes
        const void **d_ptrs = nullptr; // pattern pointer table of a table run
        size_t ptrs_cap = 0;           // bytes
        // staged layouts: per layout a run of (pattern address, first output slot)
        struct staged_group {
            uint32_t layout, offset, count;
        };
        std::vector<staged_group> sgroups;
        const void **d_sptrs = nullptr;
        uint32_t *d_sbase = nullptr;
        size_t sptrs_cap = 0, sbase_cap = 0;  // bytes
        cudaEvent_t done = nullptr;    // recorded after the launches that read this set
        bool pending = false;
    };
    static constexpr int RING = 3;
    work_set sets[RING + 1];
    int ring_next = 0;
    uint32_t src_w = 0, src_h = 0;
    int precision = EMIDA_GB_FLOAT;
    bool dbl = false;
    std::vector<layout> layouts;
    std::vector<size_class> classes;
    double *d_lstsq_all = nullptr;
    uint32_t *d_err = nullptr;
    // the fused kernels' pair queue (two words, zero between launches): every
    // class launch runs on `stream`, so one queue serves them all
    uint32_t *d_queue = nullptr;
    cudaStream_t stream = nullptr;
    // graph cache: the last captured run and what it was captured for
    cudaGraphExec_t gexec = nullptr;
    const void *g_pics = nullptr;
    uint32_t g_patterns = 0;
    std::vector<uint32_t> g_layout_of;
    double *g_offs = nullptr, *g_coefs = nullptr;
    void *g_maxes = nullptr;
    std::mutex mu;
};

namespace {

constexpr uint32_t STAGED_BATCH = 16;

size_t spec_bytes_per_roi(uint32_t n, bool dbl) { return (size_t)(n / 2 + 1) * n * (dbl ? 16 : 8); }

int grow(void **buf, size_t *cap_bytes, size_t need, size_t keep)
{
    if (need <= *cap_bytes) return EMIDA_GB_OK;
    size_t cap = std::max(need, *cap_bytes * 2);
    void *nb = nullptr;
    CK(cudaMalloc(&nb, cap));
    if (*buf && keep) CK(cudaMemcpy(nb, *buf, keep, cudaMemcpyDeviceToDevice));
    if (*buf) CK(cudaFree(*buf));
    *buf = nb;
    *cap_bytes = cap;
    return EMIDA_GB_OK;
}

void drop_graph(emida_gb_multi *m)
{
    if (m->gexec) cudaGraphExecDestroy(m->gexec);
    m->gexec = nullptr;
    m->g_layout_of.clear();
}

// Work lists of one run; returns the total ROI count.
struct staged_item {
    uint32_t pattern, layout;
    uint64_t base;  // first output slot
};
struct plan {
    std::vector<std::vector<uint4>> items;  // per class
    std::vector<staged_item> staged;
    uint64_t total = 0;
};

// Entry p reads pattern slots[p] (p itself without a slot list) of the device
// pattern array and writes its ROIs after those of entries 0..p-1.
int make_plan(emida_gb_multi *m, uint32_t patterns, const uint32_t *layout_of, plan &pl,
              const uint32_t *slots = nullptr, uint32_t arena = 0)
{
    pl.items.assign(m->classes.size(), {});
    for (uint32_t p = 0; p < patterns; ++p) {
        if (layout_of[p] >= m->layouts.size())
            return fail(EMIDA_GB_INVALID_ARGUMENT, "pattern %u: unknown layout %u", p, layout_of[p]);
        const uint32_t slot = slots ? slots[p] : p;
        if (slots && slot >= arena)
            return fail(EMIDA_GB_INVALID_ARGUMENT, "pattern %u: slot %u outside the array", p, slot);
        const auto &L = m->layouts[layout_of[p]];
        if (m->classes[L.cls].fused) {
            auto &v = pl.items[L.cls];
            for (uint32_t r = 0; r < L.n_rois; ++r)
                v.push_back(make_uint4(slot, L.roi_base + r, (uint32_t)(pl.total + r), (uint32_t)L.fitsize));
        } else {
            pl.staged.push_back(staged_item{slot, layout_of[p], pl.total});
        }
        pl.total += L.n_rois;
    }
    if (pl.total >= (1ull << 32)) return fail(EMIDA_GB_INVALID_ARGUMENT, "too many ROIs in one run");
    return EMIDA_GB_OK;
}

using work_set = emida_gb_multi::work_set;

// Host -> device copy of a work list by SM loads from the pinned staging
// buffer (over NVLink-C2C), not by the copy engine: a copy engine runs its
// copies in order, so a step's small lists would otherwise wait behind every
// pattern copy queued before them (the request loop queues whole rows).
// dst, src 16-byte aligned; bytes a multiple of 4.
__global__ void __launch_bounds__(256) k_upload(unsigned char *__restrict__ dst,
                                                const unsigned char *__restrict__ src, size_t bytes)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t n16 = bytes / 16;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride)
        reinterpret_cast<int4 *>(dst)[i] = reinterpret_cast<const int4 *>(src)[i];
    for (size_t j = n16 * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < bytes / 4; j += stride)
        reinterpret_cast<uint32_t *>(dst)[j] = reinterpret_cast<const uint32_t *>(src)[j];
}

int upload(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    const size_t n16 = (bytes + 15) / 16;
    const unsigned grid = (unsigned)std::min<size_t>(64, std::max<size_t>(1, (n16 + 255) / 256));
    k_upload<<<grid, 256, 0, st>>>(static_cast<unsigned char *>(dst), static_cast<const unsigned char *>(src),
                                   bytes);
    CK(cudaGetLastError());
    return EMIDA_GB_OK;
}

// Stages the plan's work lists in `ws` and queues their copies on m->stream,
// ahead of the launches that read them.  The set must not be read by work
// still in flight: the graph's set waits for the stream (a replay may be
// running), a ring set for the run that used it last.
int upload_plan(emida_gb_multi *m, const plan &pl, work_set &ws, bool graph_set, const void *pics,
                const void *const *ptrs = nullptr, uint32_t n_ptrs = 0)
{
    if (graph_set)
        CK(cudaStreamSynchronize(m->stream));
    else if (ws.pending)
        CK(cudaEventSynchronize(ws.done));
    ws.pending = false;
    ws.d_items.resize(m->classes.size(), nullptr);
    ws.cap.resize(m->classes.size(), 0);
    // staged patterns grouped by layout, in plan order within a layout
    ws.sgroups.clear();
    std::vector<const void *> sptrs;
    std::vector<uint32_t> sbase;
    if (!pl.staged.empty()) {
        const size_t pat_bytes = (size_t)m->src_w * m->src_h * 2;
        std::vector<std::vector<const staged_item *>> by_layout(m->layouts.size());
        std::vector<uint32_t> order;
        for (const auto &e : pl.staged) {
            if (by_layout[e.layout].empty()) order.push_back(e.layout);
            by_layout[e.layout].push_back(&e);
        }
        for (uint32_t l : order) {
            ws.sgroups.push_back({l, (uint32_t)sptrs.size(), (uint32_t)by_layout[l].size()});
            for (const staged_item *e : by_layout[l]) {
                sptrs.push_back(ptrs ? ptrs[e->pattern]
                                     : (const void *)((const char *)pics + e->pattern * pat_bytes));
                sbase.push_back((uint32_t)e->base);
            }
        }
    }
    auto up16 = [](size_t v) { return (v + 15) / 16 * 16; };
    size_t total = up16((size_t)n_ptrs * sizeof(void *)) + up16(sptrs.size() * sizeof(void *)) +
                   up16(sbase.size() * sizeof(uint32_t));
    for (const auto &v : pl.items) total += v.size() * sizeof(uint4);
    if (total > ws.h_cap) {
        if (ws.h_stage) CK(cudaFreeHost(ws.h_stage));
        ws.h_stage = nullptr;
        const size_t cap = std::max(total, 2 * ws.h_cap);
        CK(cudaMallocHost((void **)&ws.h_stage, cap));
        ws.h_cap = cap;
    }
    size_t off = 0;
    auto stage = [&](void **dst, size_t *cap, const void *src, size_t need) -> int {
        if (!need) return EMIDA_GB_OK;
        CKS(grow(dst, cap, need, 0));
        char *s = reinterpret_cast<char *>(ws.h_stage) + off;
        std::memcpy(s, src, need);
        CKS(upload(*dst, s, need, m->stream));
        off += up16(need);
        return EMIDA_GB_OK;
    };
    CKS(stage((void **)&ws.d_ptrs, &ws.ptrs_cap, ptrs, (size_t)n_ptrs * sizeof(void *)));
    CKS(stage((void **)&ws.d_sptrs, &ws.sptrs_cap, sptrs.data(), sptrs.size() * sizeof(void *)));
    CKS(stage((void **)&ws.d_sbase, &ws.sbase_cap, sbase.data(), sbase.size() * sizeof(uint32_t)));
    for (size_t c = 0; c < m->classes.size(); ++c) {
        const auto &v = pl.items[c];
        if (v.empty()) continue;
        const size_t need = v.size() * sizeof(uint4);
        CKS(grow((void **)&ws.d_items[c], &ws.cap[c], need, 0));
        char *stage = reinterpret_cast<char *>(ws.h_stage) + off;
        std::memcpy(stage, v.data(), need);
        CKS(upload(ws.d_items[c], stage, need, m->stream));
        off += need;
    }
    return EMIDA_GB_OK;
}

work_set &next_ring_set(emida_gb_multi *m)
{
    work_set &ws = m->sets[m->ring_next];
    m->ring_next = (m->ring_next + 1) % emida_gb_multi::RING;
    return ws;
}

int mark_used(emida_gb_multi *m, work_set &ws)
{
    CK(cudaEventRecord(ws.done, m->stream));
    ws.pending = true;
    return EMIDA_GB_OK;
}

// The launches of one run, on m->stream (capturable).
// `pics` is the pattern array that work-list entries index; with a pointer
// table (`table`, the host copy of ws.d_ptrs) entries index the table instead.
int launch_plan(emida_gb_multi *m, const plan &pl, const work_set &ws, const void *pics,
                uint32_t patterns, double *offs, double *coefs, void *maxes, int only_class = -1,
                int grid_override = -1, const void *const *table = nullptr)
{
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    bool on_device = false;
    if (!table) CKS(pattern_location(pics, on_device));
    // one TMA map per size class (the box is the ROI side + 8 by the ROI side)
    const bool use_tma = on_device && (m->src_w % 8) == 0 && ((uintptr_t)pics % 16) == 0 &&
                         get_encoder() != nullptr;
    // otherwise (host patterns, pattern tables) cp.async chunks, where every
    // pattern starts on a 16-byte boundary
    bool use_async = (m->src_w % 8) == 0;
    if (table)
        for (uint32_t p = 0; p < patterns && use_async; ++p) use_async = (uintptr_t)table[p] % 16 == 0;
    else
        use_async = use_async && (uintptr_t)pics % 16 == 0;
    for (size_t c = 0; c < m->classes.size(); ++c) {
        if (only_class >= 0 && (int)c != only_class) continue;
        auto &k = m->classes[c];
        if (!k.fused || pl.items[c].empty()) continue;
        fused_args a{};
        a.pics = pics;
        a.src_w = m->src_w;
        a.src_h = m->src_h;
        a.begins = k.d_begins;
        a.n_rois = 1;
        a.n_pairs = (uint32_t)pl.items[c].size();
        a.side = k.side;
        a.ref_spec = k.d_spec;
        a.hann = k.hann;
        a.twiddles = k.twiddles;
        a.lstsq = nullptr;
        a.lstsq_all = m->d_lstsq_all;
        a.fitsize = 3;
        a.offsets = offs;
        a.coefs = coefs;
        a.maxes = maxes;
        a.neigh = nullptr;
        a.err = m->d_err;
        a.items = ws.d_items[c];
        a.pattern_ptrs = table ? ws.d_ptrs : nullptr;
        a.pairs_per_cta = k.ppc;
        a.pair_queue = m->d_queue;
        a.stage = STAGE_PLAIN;
        if (use_tma) {
            const uint32_t side = k.side;
            const cuuint64_t dims[3] = {m->src_w, m->src_h, patterns};
            const cuuint64_t strides[2] = {(cuuint64_t)m->src_w * 2, (cuuint64_t)m->src_w * m->src_h * 2};
            const cuuint32_t box[3] = {(side + 14) & ~7u, fused_box_rows(k.n, side), 1};
            const cuuint32_t estr[3] = {1, 1, 1};
            if (get_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void *>(pics), dims,
                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
                a.stage = STAGE_TMA;
        }
        if (a.stage == STAGE_PLAIN && use_async) a.stage = STAGE_ASYNC;
        const int grid = grid_override >= 0 ? grid_override : k.grid ? k.grid : -m->reserve;
        CK(launch_fused(k.n, m->dbl, false, a, &map, grid, m->stream));
    }
    if (only_class >= 0) return EMIDA_GB_OK;
    // staged layouts: batches of their patterns through the staged pipeline,
    // results scattered to each pattern's output slots
    for (const auto &sg : ws.sgroups) {
        emida_gb_handle *h = m->layouts[sg.layout].h;
        for (uint32_t k = 0; k < sg.count; k += h->B) {
            const uint32_t c = std::min(h->B, sg.count - k);
            CKS(run_plain_chunk(h, nullptr, c, nullptr, nullptr, offs, coefs, m->stream,
                                ws.d_sptrs + sg.offset + k, ws.d_sbase + sg.offset + k, maxes));
        }
    }
    return EMIDA_GB_OK;
}

}  // namespace

namespace {

// The parameters of a layout's handle (reference spectra, and the staged
// pipeline for sides without a fused kernel).
emida_gb_params layout_params(const emida_gb_multi *m, const uint32_t *begins, uint32_t n_rois, uint32_t side,
                              int32_t fitsize)
{
    emida_gb_params p{};
    p.src_w = m->src_w;
    p.src_h = m->src_h;
    p.begins = begins;
    p.n_rois = n_rois;
    p.slice_w = p.slice_h = side;
    p.cross_w = p.cross_h = 2 * side - 1;
    // layouts without a fused kernel run the staged pipeline over up to
    // STAGED_BATCH of their patterns per launch sequence
    p.batch_size = fused_size_for(side, m->dbl) ? 1 : STAGED_BATCH;
    p.policy = EMIDA_GB_FFT;
    p.precision = m->precision;
    p.fitsize = fitsize;
    p.in_type = EMIDA_GB_IN_U16;
    p.mode = EMIDA_GB_MODE_AUTO;
    p.in_buffers = 1;
    return p;
}

// Handles of the given layouts at fused length n (their reference spectra
// computed from the reference pattern their current handles hold).
int class_handles(emida_gb_multi *m, const std::vector<size_t> &members, uint32_t n,
                  std::vector<emida_gb_handle *> &out)
{
    for (emida_gb_handle *h : out) emida_gb_destroy(h);
    out.clear();
    std::vector<uint16_t> ref((size_t)m->src_w * m->src_h);
    for (size_t i : members) {
        const auto &L = m->layouts[i];
        CK(cudaMemcpy(ref.data(), L.h->d_ref_in, ref.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost));
        const emida_gb_params p = layout_params(m, L.h->begins.data(), L.n_rois, L.side, L.fitsize);
        emida_gb_handle *h = nullptr;
        CKS(create_handle(&p, n, &h));
        out.push_back(h);
        CKS(emida_gb_set_reference(h, ref.data()));
    }
    return EMIDA_GB_OK;
}

// Class c's resident spectra (and twiddles, window) at fused length n, from
// `hs` (one handle per member, in member order) or, when empty, from the
// members' own handles.
int install_class_spectra(emida_gb_multi *m, size_t c, const std::vector<size_t> &members,
                          const std::vector<emida_gb_handle *> &hs, uint32_t n)
{
    auto &k = m->classes[c];
    CK(cudaStreamSynchronize(m->stream));  // no run may read the spectra being replaced
    const size_t per = spec_bytes_per_roi(n, m->dbl);
    size_t cap = k.spec_cap * spec_bytes_per_roi(k.n, m->dbl);
    CKS(grow(&k.d_spec, &cap, k.begins.size() * per, 0));
    k.spec_cap = cap / per;
    for (size_t j = 0; j < members.size(); ++j) {
        const auto &L = m->layouts[members[j]];
        emida_gb_handle *h = hs.empty() ? L.h : hs[j];
        CK(cudaMemcpy((char *)k.d_spec + (size_t)L.roi_base * per, h->d_ref_spec_cm, (size_t)L.n_rois * per,
                      cudaMemcpyDeviceToDevice));
    }
    emida_gb_handle *first = hs.empty() ? m->layouts[members.front()].h : hs.front();
    k.n = n;
    k.hann = first->d_hann_fused;
    k.twiddles = first->d_tw_row;
    return EMIDA_GB_OK;
}

}  // namespace

int emida_gb::host::multi_reserve_work(emida_gb_multi *m, uint32_t patterns)
{
    if (!m) return fail(EMIDA_GB_INVALID_ARGUMENT, "null planner");
    std::lock_guard<std::mutex> lk(m->mu);
    // the largest layout of each size class bounds a run's work list there
    std::vector<uint32_t> most(m->classes.size(), 0);
    for (const auto &L : m->layouts) most[L.cls] = std::max(most[L.cls], L.n_rois);
    // no set may be regrown under a run still reading it
    CK(cudaStreamSynchronize(m->stream));
    for (auto &ws : m->sets) {
        ws.pending = false;
        ws.d_items.resize(m->classes.size(), nullptr);
        ws.cap.resize(m->classes.size(), 0);
        size_t staging = 3 * 16 + 2 * (size_t)patterns * sizeof(void *) + (size_t)patterns * sizeof(uint32_t);
        for (size_t c = 0; c < m->classes.size(); ++c) {
            const size_t need = (size_t)patterns * most[c] * sizeof(uint4);
            if (m->classes[c].fused && need) CKS(grow((void **)&ws.d_items[c], &ws.cap[c], need, 0));
            staging += need;
        }
        CKS(grow((void **)&ws.d_ptrs, &ws.ptrs_cap, (size_t)patterns * sizeof(void *), 0));
        CKS(grow((void **)&ws.d_sptrs, &ws.sptrs_cap, (size_t)patterns * sizeof(void *), 0));
        CKS(grow((void **)&ws.d_sbase, &ws.sbase_cap, (size_t)patterns * sizeof(uint32_t), 0));
        if (staging > ws.h_cap) {
            if (ws.h_stage) CK(cudaFreeHost(ws.h_stage));
            ws.h_stage = nullptr;
            CK(cudaMallocHost((void **)&ws.h_stage, staging));
            ws.h_cap = staging;
        }
    }
    return EMIDA_GB_OK;
}

int emida_gb::host::multi_reserve_ctas(emida_gb_multi *m, int ctas)
{
    if (!m || ctas < 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "bad argument");
    std::lock_guard<std::mutex> lk(m->mu);
    m->reserve = ctas;
    drop_graph(m);  // captured with the grids chosen before
    return EMIDA_GB_OK;
}

extern "C" {

int emida_gb_multi_create(uint32_t src_w, uint32_t src_h, int32_t precision, emida_gb_multi **out)
{
    if (!out) return fail(EMIDA_GB_INVALID_ARGUMENT, "null output");
    *out = nullptr;
    if (src_w == 0 || src_h == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "empty pattern size");
    if (precision != EMIDA_GB_DOUBLE && precision != EMIDA_GB_FLOAT)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid precision %d", precision);
    auto m = std::make_unique<emida_gb_multi>();
    m->src_w = src_w;
    m->src_h = src_h;
    m->precision = precision;
    m->dbl = precision == EMIDA_GB_DOUBLE;
    std::vector<double> all(984);
    for (int s : {3, 5, 7, 9}) lstsq_matrix(s, all.data() + lstsq_offset(s));
    CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    for (auto &ws : m->sets) CK(cudaEventCreateWithFlags(&ws.done, cudaEventDisableTiming));
    CK(cudaMalloc((void **)&m->d_lstsq_all, all.size() * sizeof(double)));
    CK(cudaMemcpy(m->d_lstsq_all, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMalloc((void **)&m->d_err, sizeof(uint32_t)));
    CK(cudaMemset(m->d_err, 0, sizeof(uint32_t)));
    CK(cudaMalloc((void **)&m->d_queue, 2 * sizeof(uint32_t)));
    CK(cudaMemset(m->d_queue, 0, 2 * sizeof(uint32_t)));
    *out = m.release();
    return EMIDA_GB_OK;
}

int emida_gb_multi_add_layout(emida_gb_multi *m, const uint32_t *begins, uint32_t n_rois,
                              uint32_t side, int32_t fitsize, const uint16_t *ref,
                              uint32_t *layout_id)
{
    if (!m || !begins || !ref || !layout_id) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(m->mu);
    const emida_gb_params p = layout_params(m, begins, n_rois, side, fitsize);
    emida_gb_handle *h = nullptr;
    CKS(emida_gb_create(&p, &h));
    int st = emida_gb_set_reference(h, ref);
    if (st != EMIDA_GB_OK) {
        emida_gb_destroy(h);
        return st;
    }
    emida_gb_multi::layout L;
    L.n_rois = n_rois;
    L.side = side;
    L.fitsize = fitsize;
    L.h = h;
    // one class per ROI side (the Hann windows differ); its transform length
    // is the handle's (2 * side, or the fused length it is padded to)
    const uint32_t n = h->w2;
    int cls = -1;
    for (size_t c = 0; c < m->classes.size(); ++c)
        if (m->classes[c].side == side) cls = (int)c;
    if (cls < 0) {
        emida_gb_multi::size_class k;
        k.n = n;
        k.side = side;
        k.fused = emida_gb_resolved_mode(h) == EMIDA_GB_MODE_FUSED;
        k.hann = h->d_hann_fused;
        k.twiddles = h->d_tw_row;
        m->classes.push_back(k);
        cls = (int)m->classes.size() - 1;
    }
    L.cls = cls;
    auto &k = m->classes[cls];
    if (k.fused) {
        L.roi_base = (uint32_t)k.begins.size();
        for (uint32_t r = 0; r < n_rois; ++r) k.begins.push_back(make_uint2(begins[2 * r], begins[2 * r + 1]));
        const size_t per = spec_bytes_per_roi(n, m->dbl);
        size_t bcap = k.begins_cap * sizeof(uint2), scap = k.spec_cap * per;
        CKS(grow((void **)&k.d_begins, &bcap, k.begins.size() * sizeof(uint2), 0));
        CKS(grow(&k.d_spec, &scap, k.begins.size() * per, (size_t)L.roi_base * per));
        k.begins_cap = bcap / sizeof(uint2);
        k.spec_cap = scap / per;
        CK(cudaMemcpy(k.d_begins, k.begins.data(), k.begins.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        CK(cudaMemcpy((char *)k.d_spec + (size_t)L.roi_base * per, h->d_ref_spec_cm, (size_t)n_rois * per,
                      cudaMemcpyDeviceToDevice));
    }
    m->layouts.push_back(L);
    drop_graph(m);  // spectra or tables may have moved
    *layout_id = (uint32_t)m->layouts.size() - 1;
    return EMIDA_GB_OK;
}

int emida_gb_multi_count(const emida_gb_multi *m, uint32_t patterns, const uint32_t *layout_of,
                         uint64_t *total)
{
    if (!m || !layout_of || !total) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    uint64_t t = 0;
    for (uint32_t p = 0; p < patterns; ++p) {
        if (layout_of[p] >= m->layouts.size())
            return fail(EMIDA_GB_INVALID_ARGUMENT, "pattern %u: unknown layout %u", p, layout_of[p]);
        t += m->layouts[layout_of[p]].n_rois;
    }
    *total = t;
    return EMIDA_GB_OK;
}

int emida_gb_multi_run(emida_gb_multi *m, const void *dev_patterns, uint32_t patterns,
                       const uint32_t *layout_of, double *dev_offsets, double *dev_coefs,
                       void *dev_maxes, int use_graph)
{
    trace_range tr("emida_gb_multi_run");
    if (!m || !dev_patterns || !layout_of || !dev_offsets)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(m->mu);
    const bool same = m->gexec && m->g_pics == dev_patterns && m->g_patterns == patterns &&
                      m->g_offs == dev_offsets && m->g_coefs == dev_coefs && m->g_maxes == dev_maxes &&
                      std::equal(m->g_layout_of.begin(), m->g_layout_of.end(), layout_of) &&
                      m->g_layout_of.size() == patterns;
    if (use_graph && same) {
        CK(cudaGraphLaunch(m->gexec, m->stream));
        return EMIDA_GB_OK;
    }
    plan pl;
    CKS(make_plan(m, patterns, layout_of, pl));
    if (!use_graph) {
        work_set &ws = next_ring_set(m);
        CKS(upload_plan(m, pl, ws, false, dev_patterns));
        CKS(launch_plan(m, pl, ws, dev_patterns, patterns, dev_offsets, dev_coefs, dev_maxes));
        return mark_used(m, ws);
    }
    drop_graph(m);  // the graph's work lists are about to be overwritten
    work_set &gs = m->sets[emida_gb_multi::RING];
    CKS(upload_plan(m, pl, gs, true, dev_patterns));
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeRelaxed));
    int st = launch_plan(m, pl, gs, dev_patterns, patterns, dev_offsets, dev_coefs, dev_maxes);
    cudaError_t e = cudaStreamEndCapture(m->stream, &graph);
    if (st != EMIDA_GB_OK) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return st;
    }
    CK(e);
    e = cudaGraphInstantiate(&m->gexec, graph, 0);
    cudaGraphDestroy(graph);
    CK(e);
    m->g_pics = dev_patterns;
    m->g_patterns = patterns;
    m->g_offs = dev_offsets;
    m->g_coefs = dev_coefs;
    m->g_maxes = dev_maxes;
    m->g_layout_of.assign(layout_of, layout_of + patterns);
    CK(cudaGraphLaunch(m->gexec, m->stream));
    return EMIDA_GB_OK;
}

int emida_gb_multi_run_slots(emida_gb_multi *m, const void *dev_patterns, uint32_t arena,
                             uint32_t patterns, const uint32_t *slots, const uint32_t *layout_of,
                             double *dev_offsets, double *dev_coefs, void *dev_maxes)
{
    trace_range tr("emida_gb_multi_run_slots");
    if (!m || !dev_patterns || !slots || !layout_of || !dev_offsets)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(m->mu);
    plan pl;
    CKS(make_plan(m, patterns, layout_of, pl, slots, arena));
    work_set &ws = next_ring_set(m);
    CKS(upload_plan(m, pl, ws, false, dev_patterns));
    CKS(launch_plan(m, pl, ws, dev_patterns, arena, dev_offsets, dev_coefs, dev_maxes));
    return mark_used(m, ws);
}

int emida_gb_multi_run_table(emida_gb_multi *m, const void *const *patterns, uint32_t n,
                             const uint32_t *layout_of, double *dev_offsets, double *dev_coefs,
                             void *dev_maxes)
{
    trace_range tr("emida_gb_multi_run_table");
    if (!m || !patterns || !layout_of || !dev_offsets)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    for (uint32_t p = 0; p < n; ++p) {
        bool on_device = true;
        if (!patterns[p]) return fail(EMIDA_GB_INVALID_ARGUMENT, "pattern %u: null pointer", p);
        CKS(pattern_location(patterns[p], on_device));
    }
    std::lock_guard<std::mutex> lk(m->mu);
    plan pl;
    CKS(make_plan(m, n, layout_of, pl));
    work_set &ws = next_ring_set(m);
    CKS(upload_plan(m, pl, ws, false, nullptr, patterns, n));
    CKS(launch_plan(m, pl, ws, nullptr, n, dev_offsets, dev_coefs, dev_maxes, -1, -1, patterns));
    return mark_used(m, ws);
}

void *emida_gb_multi_stream(emida_gb_multi *m) { return m ? (void *)m->stream : nullptr; }

int emida_gb_multi_synchronize(emida_gb_multi *m)
{
    if (!m) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(m->stream));
    uint32_t err = 0;
    CK(cudaMemcpy(&err, m->d_err, sizeof err, cudaMemcpyDeviceToHost));
    if (err) {
        CK(cudaMemset(m->d_err, 0, sizeof err));
        return fail(EMIDA_GB_DEVICE_CHECK, "device check failed (flags 0x%x)", err);
    }
    return EMIDA_GB_OK;
}

int emida_gb_multi_autotune(emida_gb_multi *m, const void *dev_patterns, uint32_t patterns,
                            const uint32_t *layout_of, double *dev_offsets, char *report,
                            size_t report_len)
{
    if (!m || !dev_patterns || !layout_of || !dev_offsets)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(m->mu);
    plan pl;
    CKS(make_plan(m, patterns, layout_of, pl));
    work_set &ws = next_ring_set(m);
    CKS(upload_plan(m, pl, ws, false, dev_patterns));
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    std::string rep;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    auto time_grid = [&](size_t c, int grid, float &ms) -> int {
        CKS(launch_plan(m, pl, ws, dev_patterns, patterns, dev_offsets, nullptr, nullptr, (int)c, grid));
        CK(cudaEventRecord(a, m->stream));
        for (int r = 0; r < 3; ++r)
            CKS(launch_plan(m, pl, ws, dev_patterns, patterns, dev_offsets, nullptr, nullptr, (int)c, grid));
        CK(cudaEventRecord(b, m->stream));
        CK(cudaEventSynchronize(b));
        CK(cudaEventElapsedTime(&ms, a, b));
        ms /= 3;
        return EMIDA_GB_OK;
    };
    int st = EMIDA_GB_OK;
    for (size_t c = 0; c < m->classes.size() && st == EMIDA_GB_OK; ++c) {
        auto &k = m->classes[c];
        if (!k.fused || pl.items[c].empty()) continue;
        // tile shapes: the transform lengths that hold the ROI (its own and the
        // next one, which zero-pads it further), each with 1..6 CTAs per SM
        std::vector<uint32_t> lens;
        for (uint32_t n : {64u, 96u, 128u, 192u, 256u})
            if (n >= 2 * k.side && fused_supported(n, m->dbl) && lens.size() < 2) lens.push_back(n);
        std::vector<size_t> members;
        for (size_t i = 0; i < m->layouts.size(); ++i)
            if (m->layouts[i].cls == (int)c) members.push_back(i);
        const uint32_t n0 = k.n;
        float best = 1e30f;
        int best_grid = 0;
        uint32_t best_n = n0, best_ppc = 0;
        std::string tried;
        std::vector<emida_gb_handle *> alt;  // the other length's handles, one per member
        for (uint32_t n : lens) {
            if (n != n0) {
                st = class_handles(m, members, n, alt);
                if (st == EMIDA_GB_OK) st = install_class_spectra(m, c, members, alt, n);
            } else if (k.n != n0) {
                st = install_class_spectra(m, c, members, {}, n0);  // the members' own length again
            }
            if (st != EMIDA_GB_OK) break;
            // tile shapes of this length: pairs per CTA (the FP32 96-point
            // kernel is built with 4, 2 and 1)
            std::vector<uint32_t> ppcs = {0};
            if (n == 96 && !m->dbl) ppcs = {4, 2, 1};
            for (uint32_t ppc : ppcs) {
                k.ppc = ppc;
                float nbest = 1e30f;
                int ngrid = 0;
                for (int per_sm = 1; per_sm <= 6 && st == EMIDA_GB_OK; ++per_sm) {
                    float ms = 0;
                    st = time_grid(c, per_sm * sms, ms);
                    if (st == EMIDA_GB_OK && ms < nbest * 0.98f) {
                        nbest = ms;
                        ngrid = per_sm * sms;
                    }
                }
                if (st != EMIDA_GB_OK) break;
                char t[64];
                if (ppc)
                    snprintf(t, sizeof t, "%sn=%u/%u per CTA %.3f ms", tried.empty() ? "" : ", ", n, ppc, nbest);
                else
                    snprintf(t, sizeof t, "%sn=%u %.3f ms", tried.empty() ? "" : ", ", n, nbest);
                tried += t;
                if (nbest < best * 0.98f) {
                    best = nbest;
                    best_grid = ngrid;
                    best_n = n;
                    best_ppc = ppc;
                }
            }
            k.ppc = 0;
            if (st != EMIDA_GB_OK) break;
        }
        // keep the winning length's spectra and handles
        std::vector<emida_gb_handle *> orig;
        for (size_t i : members) orig.push_back(m->layouts[i].h);
        if (st == EMIDA_GB_OK && best_n != n0) {
            for (size_t j = 0; j < members.size(); ++j) m->layouts[members[j]].h = alt[j];
            alt.swap(orig);
        }
        int st2 = install_class_spectra(m, c, members, {}, best_n);
        if (st == EMIDA_GB_OK) st = st2;
        CK(cudaStreamSynchronize(m->stream));
        for (emida_gb_handle *h : alt) emida_gb_destroy(h);
        if (st != EMIDA_GB_OK) break;
        k.grid = best_grid;
        k.ppc = best_ppc;
        char line[256];
        // the default with the runner's pair queue: 2 at 96 points (FP32), else 1
        const uint32_t shown_ppc = k.ppc ? k.ppc : (k.n == 96 && !m->dbl ? 2u : 1u);
        snprintf(line, sizeof line, "side %u (n=%u): %zu pairs, grid %d (%d per SM), %u pair%s per CTA, %.3f ms [%s]\n",
                 k.side, k.n, pl.items[c].size(), best_grid, best_grid / std::max(1, sms), shown_ppc,
                 shown_ppc == 1 ? "" : "s", best, tried.c_str());
        rep += line;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    CKS(mark_used(m, ws));
    drop_graph(m);  // captured with the grids chosen before
    if (report && report_len) {
        std::strncpy(report, rep.c_str(), report_len - 1);
        report[report_len - 1] = 0;
    }
    return st;
}

void emida_gb_multi_destroy(emida_gb_multi *m)
{
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    drop_graph(m);
    for (auto &k : m->classes) {
        if (k.d_begins) cudaFree(k.d_begins);
        if (k.d_spec) cudaFree(k.d_spec);
    }
    for (auto &ws : m->sets) {
        for (uint4 *p : ws.d_items)
            if (p) cudaFree(p);
        if (ws.d_ptrs) cudaFree(ws.d_ptrs);
        if (ws.d_sptrs) cudaFree(ws.d_sptrs);
        if (ws.d_sbase) cudaFree(ws.d_sbase);
        if (ws.h_stage) cudaFreeHost(ws.h_stage);
        if (ws.done) cudaEventDestroy(ws.done);
    }
    for (auto &L : m->layouts) emida_gb_destroy(L.h);
    if (m->d_lstsq_all) cudaFree(m->d_lstsq_all);
    if (m->d_err) cudaFree(m->d_err);
    if (m->d_queue) cudaFree(m->d_queue);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

}  // extern "C"
