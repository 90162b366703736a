// server.cu -- a request loop over the multi-layout planner.  A request is a
// scan row: n patterns of one size on one registered ROI layout (reference
// spectra resident per layout).  A pinned row on a layout whose ROIs cover at
// most half of the pattern is read in place by the kernels; any other row is
// admitted while the device pattern arena of its size has room for all its
// patterns (admission by free HBM) and copied in on its own stream, chunk by
// chunk, only its ROI row bands.  Steps of up to step_patterns patterns are
// filled from the oldest admitted rows first (continuous batching): a row that
// arrives while others run joins the next step that has room, so its work
// overlaps theirs on the device.  Each pattern size has its own planner and
// streams, so their steps overlap too.  The reference's counterpart is the
// load / GPU / finalize thread pipeline of src/process_files.hpp:79-237, which
// runs one layout and one row at a time.
#include <algorithm>
#include <array>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#include "handle.cuh"

using namespace emida_gb;
using namespace emida_gb::host;

namespace {

using clock_t_ = std::chrono::steady_clock;
constexpr uint32_t COPY_CHUNK = 16;
// Chunks of copied rows queued on a pool's copy stream at a time (about 1 ms
// of copies at 1024^2): enough to keep the copy engine busy between polls of
// the loop, few enough that queuing them never blocks the loop (a full driver
// queue would hold it, and with it every submit, for the copies' duration).
constexpr uint32_t COPY_WINDOW = 8;
// CTAs of the SM copies of a row's bands: host reads over NVLink-C2C reach the
// link's rate from 16 CTAs; the steps' one-wave launches leave that many CTA
// slots free so that the copy of the next chunk runs beside them.
constexpr int COPY_CTAS = 16;

struct request {
    uint64_t id = 0;
    uint32_t layout = 0, pool = 0, n = 0, rois = 0;
    const uint16_t *host = nullptr;
    std::vector<uint32_t> slots;
    uint32_t next = 0, done = 0;  // patterns scheduled / finished
    std::vector<double> offsets, coefs;
    // one event per COPY_CHUNK patterns copied in (queued so far): steps take a
    // row's patterns as soon as their chunk has landed, not when the whole row has
    std::vector<cudaEvent_t> chunks;
    uint32_t landed_chunks = 0;
    // read in place from the caller's pinned rows by the kernels: no arena
    // slots, no copy, computable from the moment it is admitted
    bool in_place = false;
    bool admitted = false, complete = false;
    int status = EMIDA_GB_OK;
    // when the row was submitted, admitted, had its first and its last step
    // launched, and completed (its last step's results handed over)
    clock_t_::time_point t_submit, t_admit, t_first_launch, t_last_launch, t_done;
    bool launched = false;
};

struct step {
    struct part {
        request *r;
        uint32_t first, count;  // patterns of the request
        uint64_t out;           // first output ROI of the part in this step
    };
    std::vector<part> parts;
    std::vector<uint32_t> slots;
    uint64_t rois = 0;
    double *d_offs = nullptr, *d_coefs = nullptr, *h_offs = nullptr, *h_coefs = nullptr;
    size_t cap = 0;  // ROIs
    cudaEvent_t done = nullptr;
    bool busy = false;
};

struct pool {
    uint32_t w = 0, h = 0;
    emida_gb_multi *m = nullptr;
    uint16_t *arena = nullptr;
    uint32_t slots = 0;
    std::vector<uint32_t> free_slots;
    cudaStream_t copy = nullptr, out = nullptr;
    std::deque<request *> pending;
    std::vector<request *> active;
    uint32_t max_rois = 0;  // largest layout of this pattern size
    step steps[2];
};

}  // namespace

struct emida_gb_server {
    int precision = EMIDA_GB_FLOAT;
    uint64_t budget = 0;
    uint32_t step_patterns = 64;
    std::vector<std::unique_ptr<pool>> pools;
    struct layout_ref {
        uint32_t pool, id, rois;
        bool sparse;  // ROIs cover at most half of the pattern: rows may be read in place
        std::vector<std::pair<uint32_t, uint32_t>> bands;  // (first row, rows) holding ROI pixels
        // the bands as (first 16-byte chunk, chunks) runs of a pattern, for SM
        // copies (null when a pattern row is not a whole number of chunks)
        uint2 *d_runs = nullptr;
        uint32_t n_runs = 0;
    };
    std::vector<layout_ref> layouts;
    std::map<uint64_t, std::unique_ptr<request>> requests;
    uint64_t next_id = 1;
    std::vector<double> latencies;  // ms, completed rows
    // per completed row: patterns, then ms from submission to admission, to
    // its first step's launch, to its last step's launch, to completion
    std::vector<std::array<double, 5>> traces;
    uint64_t pairs_done = 0;
    clock_t_::time_point t_first;
    bool started = false;
    std::mutex mu;
    std::condition_variable cv;  // submissions and completions
    std::thread loop;
    bool stop = false;
    int error = EMIDA_GB_OK;
    std::string error_msg;
    // which pinned rows the kernels read in place: 0 none (default: rows are
    // copied into the arena, by SM loads where their alignment allows), 1
    // rows of sparse layouts, 2 every pinned row
    int zero_copy = 0;
};

namespace {

int admit(emida_gb_server *, pool &p)
{
    while (!p.pending.empty()) {
        request *r = p.pending.front();
        if (r->in_place) {
            p.pending.pop_front();
            r->admitted = true;
            r->t_admit = clock_t_::now();
            p.active.push_back(r);
            continue;
        }
        if (p.free_slots.size() < r->n) break;  // wait for slots: rows are admitted whole
        p.pending.pop_front();
        r->slots.assign(p.free_slots.end() - r->n, p.free_slots.end());
        p.free_slots.resize(p.free_slots.size() - r->n);
        std::sort(r->slots.begin(), r->slots.end());  // consecutive slots copy as one
        r->admitted = true;
        r->t_admit = clock_t_::now();
        p.active.push_back(r);
    }
    return EMIDA_GB_OK;
}

// Queues the copies of admitted rows, oldest row first, chunk by chunk, while
// fewer than COPY_WINDOW chunks are on their way.
int issue_copies(emida_gb_server *sv, pool &p)
{
    uint32_t in_flight = 0;
    for (request *r : p.active) {
        while (r->landed_chunks < r->chunks.size() &&
               cudaEventQuery(r->chunks[r->landed_chunks]) == cudaSuccess)
            ++r->landed_chunks;
        in_flight += (uint32_t)r->chunks.size() - r->landed_chunks;
    }
    const size_t row = (size_t)p.w * 2, pat = row * p.h;
    for (request *r : p.active) {
        if (r->in_place) continue;
        const auto &L = sv->layouts[r->layout];
        const auto &bands = L.bands;
        // pinned, 16-byte aligned rows of whole-chunk pattern rows: SM copies
        // beside the running steps; otherwise the copy engine
        const bool sm_copy = L.d_runs && (uintptr_t)r->host % 16 == 0;
        while (in_flight < COPY_WINDOW && r->chunks.size() * COPY_CHUNK < r->n) {
            const uint32_t c0 = (uint32_t)r->chunks.size() * COPY_CHUNK;
            const uint32_t c1 = std::min(r->n, c0 + COPY_CHUNK);
            for (uint32_t a = c0; a < c1;) {
                uint32_t b = a + 1;
                while (b < c1 && r->slots[b] == r->slots[b - 1] + 1) ++b;
                // patterns a..b-1 go to consecutive slots: one pitched copy per ROI row band
                const char *src = reinterpret_cast<const char *>(r->host) + a * pat;
                char *dst = reinterpret_cast<char *>(p.arena) + r->slots[a] * pat;
                if (sm_copy)
                    CK(run_copy_bands(src, dst, L.d_runs, L.n_runs, pat / 16, b - a, COPY_CTAS, 0, p.copy));
                else
                    for (const auto &bd : bands)
                        CK(cudaMemcpy2DAsync(dst + bd.first * row, pat, src + bd.first * row, pat,
                                             bd.second * row, b - a, cudaMemcpyHostToDevice, p.copy));
                a = b;
            }
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            r->chunks.push_back(e);
            CK(cudaEventRecord(e, p.copy));
            ++in_flight;
        }
        if (in_flight >= COPY_WINDOW) break;
    }
    return EMIDA_GB_OK;
}

int ensure_step_buffers(step &st, size_t rois)
{
    if (rois <= st.cap) return EMIDA_GB_OK;
    if (st.d_offs) cudaFree(st.d_offs);
    if (st.d_coefs) cudaFree(st.d_coefs);
    if (st.h_offs) cudaFreeHost(st.h_offs);
    if (st.h_coefs) cudaFreeHost(st.h_coefs);
    st.d_offs = st.d_coefs = st.h_offs = st.h_coefs = nullptr;
    const size_t cap = std::max(rois, 2 * st.cap);
    CK(cudaMalloc((void **)&st.d_offs, cap * 2 * sizeof(double)));
    CK(cudaMalloc((void **)&st.d_coefs, cap * 6 * sizeof(double)));
    CK(cudaMallocHost((void **)&st.h_offs, cap * 2 * sizeof(double)));
    CK(cudaMallocHost((void **)&st.h_coefs, cap * 6 * sizeof(double)));
    st.cap = cap;
    if (!st.done) CK(cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming));
    return EMIDA_GB_OK;
}

// Builds and queues one step from the rows whose patterns are on the device.
// While the pool's other step keeps the GPU busy, a step that would be
// short of step_patterns waits for more copied patterns to land (when more
// are on their way), so that copies slower than the path do not cut the work
// into small, tail-heavy launches.
int launch_step(emida_gb_server *sv, pool &p, step &st, bool other_busy)
{
    if (other_busy) {
        uint32_t avail = 0;
        bool more_coming = false;
        for (request *r : p.active) {
            if (r->next >= r->n) continue;
            while (r->landed_chunks < r->chunks.size() &&
                   cudaEventQuery(r->chunks[r->landed_chunks]) == cudaSuccess)
                ++r->landed_chunks;
            const uint32_t landed = r->in_place ? r->n : std::min(r->n, r->landed_chunks * COPY_CHUNK);
            if (landed > r->next) avail += landed - r->next;
            more_coming |= landed < r->n;
        }
        if (more_coming && avail < sv->step_patterns) return EMIDA_GB_OK;
    }
    st.parts.clear();
    st.slots.clear();
    std::vector<uint32_t> layout_of;
    std::vector<const void *> ptrs;
    bool any_in_place = false;
    const size_t pat_elems = (size_t)p.w * p.h;
    st.rois = 0;
    uint32_t budget = sv->step_patterns;
    // oldest admitted rows first: a row's latency is its own work plus the
    // rows ahead of it, and a row that arrives meanwhile fills what is left
    for (size_t k = 0; k < p.active.size() && budget; ++k) {
        request *r = p.active[k];
        if (r->next >= r->n) continue;
        while (r->landed_chunks < r->chunks.size() &&
               cudaEventQuery(r->chunks[r->landed_chunks]) == cudaSuccess)
            ++r->landed_chunks;
        const uint32_t landed = r->in_place ? r->n : std::min(r->n, r->landed_chunks * COPY_CHUNK);
        if (landed <= r->next) continue;
        const uint32_t take = std::min(landed - r->next, budget);
        st.parts.push_back(step::part{r, r->next, take, st.rois});
        for (uint32_t i = 0; i < take; ++i) {
            const uint32_t k = r->next + i;
            const uint32_t slot = r->in_place ? 0 : r->slots[k];
            st.slots.push_back(slot);
            ptrs.push_back(r->in_place ? (const void *)(r->host + k * pat_elems)
                                       : (const void *)(p.arena + slot * pat_elems));
            layout_of.push_back(sv->layouts[r->layout].id);
        }
        any_in_place |= r->in_place;
        st.rois += (uint64_t)take * r->rois;
        r->next += take;
        budget -= take;
    }
    if (st.parts.empty()) return EMIDA_GB_OK;
    trace_range tr("server step");
    // sized once for the largest step this pool can build (a regrow frees
    // device memory, which waits for the whole device)
    CKS(ensure_step_buffers(st, std::max<size_t>(st.rois, (size_t)sv->step_patterns * p.max_rois)));
    if (any_in_place)
        CKS(emida_gb_multi_run_table(p.m, ptrs.data(), (uint32_t)ptrs.size(), layout_of.data(), st.d_offs,
                                     st.d_coefs, nullptr));
    else
        CKS(emida_gb_multi_run_slots(p.m, p.arena, p.slots, (uint32_t)st.slots.size(), st.slots.data(),
                                     layout_of.data(), st.d_offs, st.d_coefs, nullptr));
    const auto now = clock_t_::now();
    for (const auto &part : st.parts) {
        if (!part.r->launched) part.r->t_first_launch = now;
        part.r->launched = true;
        part.r->t_last_launch = now;
    }
    cudaStream_t ms = (cudaStream_t)emida_gb_multi_stream(p.m);
    CK(cudaEventRecord(st.done, ms));
    CK(cudaStreamWaitEvent(p.out, st.done, 0));
    CK(cudaMemcpyAsync(st.h_offs, st.d_offs, st.rois * 2 * sizeof(double), cudaMemcpyDeviceToHost, p.out));
    CK(cudaMemcpyAsync(st.h_coefs, st.d_coefs, st.rois * 6 * sizeof(double), cudaMemcpyDeviceToHost, p.out));
    CK(cudaEventRecord(st.done, p.out));
    st.busy = true;
    return EMIDA_GB_OK;
}

// Hands a finished step's results to its rows; frees their arena slots.
void retire_step(emida_gb_server *sv, pool &p, step &st)
{
    trace_range tr("server retire");
    for (const auto &part : st.parts) {
        request *r = part.r;
        const size_t n = (size_t)part.count * r->rois;
        const size_t at = (size_t)part.first * r->rois;
        std::memcpy(r->offsets.data() + 2 * at, st.h_offs + 2 * part.out, n * 2 * sizeof(double));
        std::memcpy(r->coefs.data() + 6 * at, st.h_coefs + 6 * part.out, n * 6 * sizeof(double));
        if (!r->in_place)
            for (uint32_t i = 0; i < part.count; ++i) p.free_slots.push_back(r->slots[part.first + i]);
        r->done += part.count;
        sv->pairs_done += n;
        if (r->done == r->n) {
            r->complete = true;
            r->t_done = clock_t_::now();
            auto ms = [&](clock_t_::time_point t) {
                return std::chrono::duration<double, std::milli>(t - r->t_submit).count();
            };
            sv->latencies.push_back(ms(r->t_done));
            sv->traces.push_back({(double)r->n, ms(r->t_admit), ms(r->t_first_launch), ms(r->t_last_launch),
                                  ms(r->t_done)});
            p.active.erase(std::find(p.active.begin(), p.active.end(), r));
            for (cudaEvent_t e : r->chunks) cudaEventDestroy(e);
            r->chunks.clear();
        }
    }
    st.parts.clear();
    st.busy = false;
}

void server_loop(emida_gb_server *sv)
{
    std::unique_lock<std::mutex> lk(sv->mu);
    while (!sv->stop) {
        bool progress = false;
        for (auto &pp : sv->pools) {
            pool &p = *pp;
            for (auto &st : p.steps)
                if (st.busy && cudaEventQuery(st.done) == cudaSuccess) {
                    retire_step(sv, p, st);
                    progress = true;
                }
            int rc = admit(sv, p);
            if (rc == EMIDA_GB_OK) rc = issue_copies(sv, p);
            for (int k = 0; k < 2; ++k) {
                step &st = p.steps[k];
                if (rc == EMIDA_GB_OK && !st.busy && !p.active.empty())
                    rc = launch_step(sv, p, st, p.steps[1 - k].busy);
            }
            if (rc != EMIDA_GB_OK) {
                // a failed launch fails the rows it would have served
                sv->error = rc;
                sv->error_msg = emida_gb_last_error();
                for (request *r : p.active) {
                    r->status = rc;
                    r->complete = true;
                }
                p.active.clear();
                progress = true;
            }
        }
        if (progress) sv->cv.notify_all();
        bool busy = false;
        for (auto &pp : sv->pools)
            busy |= !pp->active.empty() || !pp->pending.empty();
        if (busy)
            sv->cv.wait_for(lk, std::chrono::microseconds(50));
        else
            sv->cv.wait_for(lk, std::chrono::milliseconds(20));
    }
}

}  // namespace

extern "C" {

int emida_gb_server_create(int32_t precision, uint64_t hbm_bytes, uint32_t step_patterns,
                           emida_gb_server **out)
{
    if (!out) return fail(EMIDA_GB_INVALID_ARGUMENT, "null output");
    *out = nullptr;
    if (precision != EMIDA_GB_DOUBLE && precision != EMIDA_GB_FLOAT)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid precision %d", precision);
    if (step_patterns == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "step_patterns must be > 0");
    auto sv = std::make_unique<emida_gb_server>();
    sv->precision = precision;
    sv->budget = hbm_bytes;
    sv->step_patterns = step_patterns;
    sv->loop = std::thread(server_loop, sv.get());
    *out = sv.release();
    return EMIDA_GB_OK;
}

int emida_gb_server_add_layout(emida_gb_server *sv, uint32_t src_w, uint32_t src_h,
                               const uint32_t *begins, uint32_t n_rois, uint32_t side,
                               int32_t fitsize, const uint16_t *ref, uint32_t *layout_id)
{
    if (!sv || !layout_id) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    uint32_t pi = 0;
    while (pi < sv->pools.size() && !(sv->pools[pi]->w == src_w && sv->pools[pi]->h == src_h)) ++pi;
    if (pi == sv->pools.size()) {
        auto p = std::make_unique<pool>();
        p->w = src_w;
        p->h = src_h;
        const size_t bytes = (size_t)src_w * src_h * 2;
        p->slots = (uint32_t)std::min<uint64_t>(sv->budget / bytes, 1u << 20);
        if (p->slots == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "the HBM budget holds no pattern");
        CKS(emida_gb_multi_create(src_w, src_h, sv->precision, &p->m));
        CK(cudaMalloc((void **)&p->arena, (size_t)p->slots * bytes));
        for (uint32_t s = 0; s < p->slots; ++s) p->free_slots.push_back(p->slots - 1 - s);
        // copies go first: their CTAs are dispatched ahead of a step's pending CTAs
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CK(cudaStreamCreateWithPriority(&p->copy, cudaStreamNonBlocking, greatest));
        CKS(multi_reserve_ctas(p->m, COPY_CTAS));
        CK(cudaStreamCreateWithFlags(&p->out, cudaStreamNonBlocking));
        sv->pools.push_back(std::move(p));
    }
    uint32_t id = 0;
    CKS(emida_gb_multi_add_layout(sv->pools[pi]->m, begins, n_rois, side, fitsize, ref, &id));
    const bool sparse = 2 * (uint64_t)n_rois * side * side <= (uint64_t)src_w * src_h;
    // merged row bands of the ROIs: a copied row moves only these
    std::vector<std::pair<uint32_t, uint32_t>> iv, bands;
    for (uint32_t r = 0; r < n_rois; ++r) iv.push_back({begins[2 * r + 1], begins[2 * r + 1] + side});
    std::sort(iv.begin(), iv.end());
    for (const auto &v : iv) {
        if (!bands.empty() && v.first <= bands.back().second)
            bands.back().second = std::max(bands.back().second, v.second);
        else
            bands.push_back(v);
    }
    for (auto &b : bands) b.second -= b.first;
    emida_gb_server::layout_ref L{pi, id, n_rois, sparse, bands};
    if (((size_t)src_w * 2) % 16 == 0) {
        const uint32_t row16 = src_w * 2 / 16;
        std::vector<uint2> runs;
        for (const auto &b : bands) runs.push_back(make_uint2(b.first * row16, b.second * row16));
        CK(cudaMalloc((void **)&L.d_runs, runs.size() * sizeof(uint2)));
        CK(cudaMemcpy(L.d_runs, runs.data(), runs.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        L.n_runs = (uint32_t)runs.size();
    }
    sv->layouts.push_back(std::move(L));
    pool &pp = *sv->pools[pi];
    pp.max_rois = std::max(pp.max_rois, n_rois);
    // sized now for the largest step, so that serving allocates and frees
    // nothing (a free waits for the whole device)
    CKS(multi_reserve_work(pp.m, sv->step_patterns));
    for (auto &st : pp.steps) CKS(ensure_step_buffers(st, (size_t)sv->step_patterns * pp.max_rois));
    *layout_id = (uint32_t)sv->layouts.size() - 1;
    return EMIDA_GB_OK;
}

int emida_gb_server_submit(emida_gb_server *sv, uint32_t layout_id, const uint16_t *patterns,
                           uint32_t n, uint64_t *request_id)
{
    if (!sv || !patterns || !request_id || n == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "bad argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    if (layout_id >= sv->layouts.size()) return fail(EMIDA_GB_INVALID_ARGUMENT, "unknown layout %u", layout_id);
    const auto &L = sv->layouts[layout_id];
    pool &p = *sv->pools[L.pool];
    bool in_place = false;
    if (sv->zero_copy == 2 || (sv->zero_copy == 1 && L.sparse)) {
        cudaPointerAttributes pa{};
        CK(cudaPointerGetAttributes(&pa, patterns));
        in_place = pa.type == cudaMemoryTypeHost;
    }
    if (!in_place && n > p.slots)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "a row of %u patterns exceeds the %u-pattern arena", n, p.slots);
    auto r = std::make_unique<request>();
    r->in_place = in_place;
    r->id = sv->next_id++;
    r->layout = layout_id;
    r->pool = L.pool;
    r->n = n;
    r->rois = L.rois;
    r->host = patterns;
    r->offsets.assign((size_t)n * L.rois * 2, 0.0);
    r->coefs.assign((size_t)n * L.rois * 6, 0.0);
    r->t_submit = clock_t_::now();
    if (!sv->started) {
        sv->started = true;
        sv->t_first = r->t_submit;
    }
    p.pending.push_back(r.get());
    *request_id = r->id;
    sv->requests[r->id] = std::move(r);
    sv->cv.notify_all();
    return EMIDA_GB_OK;
}

int emida_gb_server_set_zero_copy(emida_gb_server *sv, int enable)
{
    if (!sv) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    if (enable < 0 || enable > 2) return fail(EMIDA_GB_INVALID_ARGUMENT, "zero-copy level %d not in 0..2", enable);
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->zero_copy = enable;
    return EMIDA_GB_OK;
}

int emida_gb_server_wait(emida_gb_server *sv, uint64_t request_id, double *offsets, double *coefs,
                         double *latency_ms)
{
    if (!sv) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(request_id);
    if (it == sv->requests.end())
        return fail(EMIDA_GB_INVALID_ARGUMENT, "unknown request %llu", (unsigned long long)request_id);
    request *r = it->second.get();
    sv->cv.wait(lk, [&] { return r->complete; });
    const int st = r->status;
    if (st == EMIDA_GB_OK) {
        if (offsets) std::memcpy(offsets, r->offsets.data(), r->offsets.size() * sizeof(double));
        if (coefs) std::memcpy(coefs, r->coefs.data(), r->coefs.size() * sizeof(double));
        if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    }
    sv->requests.erase(it);
    if (st != EMIDA_GB_OK) return fail(st, "request failed: %s", sv->error_msg.c_str());
    return EMIDA_GB_OK;
}

int emida_gb_server_stats(emida_gb_server *sv, double *p50_ms, double *p99_ms, double *pairs_per_s,
                          uint64_t *completed)
{
    if (!sv) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    std::vector<double> l = sv->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        const size_t i = std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5));
        return l[i];
    };
    if (p50_ms) *p50_ms = pct(0.50);
    if (p99_ms) *p99_ms = pct(0.99);
    if (completed) *completed = l.size();
    if (pairs_per_s) {
        const double s = sv->started ? std::chrono::duration<double>(clock_t_::now() - sv->t_first).count() : 0;
        *pairs_per_s = s > 0 ? sv->pairs_done / s : 0;
    }
    return EMIDA_GB_OK;
}

int emida_gb_server_trace(emida_gb_server *sv, double *rows, uint64_t capacity, uint64_t *count)
{
    if (!sv || !count) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->traces.size();
    if (rows)
        for (uint64_t i = 0; i < sv->traces.size() && i < capacity; ++i)
            std::memcpy(rows + 5 * i, sv->traces[i].data(), 5 * sizeof(double));
    return EMIDA_GB_OK;
}

int emida_gb_server_reset_stats(emida_gb_server *sv)
{
    if (!sv) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->latencies.clear();
    sv->traces.clear();
    sv->pairs_done = 0;
    sv->started = false;
    return EMIDA_GB_OK;
}

void emida_gb_server_destroy(emida_gb_server *sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->cv.notify_all();
    }
    if (sv->loop.joinable()) sv->loop.join();
    for (auto &pp : sv->pools)
        if (pp->copy) cudaStreamSynchronize(pp->copy);
    for (auto &kv : sv->requests)
        for (cudaEvent_t e : kv.second->chunks) cudaEventDestroy(e);
    for (auto &L : sv->layouts)
        if (L.d_runs) cudaFree(L.d_runs);
    for (auto &pp : sv->pools) {
        pool &p = *pp;
        if (p.m) emida_gb_multi_synchronize(p.m);
        if (p.copy) cudaStreamSynchronize(p.copy);
        if (p.out) cudaStreamSynchronize(p.out);
        for (auto &st : p.steps) {
            if (st.d_offs) cudaFree(st.d_offs);
            if (st.d_coefs) cudaFree(st.d_coefs);
            if (st.h_offs) cudaFreeHost(st.h_offs);
            if (st.h_coefs) cudaFreeHost(st.h_coefs);
            if (st.done) cudaEventDestroy(st.done);
        }
        if (p.arena) cudaFree(p.arena);
        if (p.copy) cudaStreamDestroy(p.copy);
        if (p.out) cudaStreamDestroy(p.out);
        emida_gb_multi_destroy(p.m);
    }
    delete sv;
}

}  // extern "C"
