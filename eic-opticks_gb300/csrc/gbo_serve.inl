// gbo_serve.inl : continuous-batching event server over one engine (included at the end of gbo_engine.cu).
//
// The reference runs one event at a time: G4CXOpticks::simulate uploads the gensteps, launches, synchronises and
// gathers hits before returning (qudarap/QSim.cc:428-631, CSGOptiX/CSGOptiX.cc:1172-1174); its service layer
// (CSGOptiX/CSGOptiXService.h) serves one request at a time.  Here producer threads submit events and go on; a
// worker thread packs whatever events are waiting into one launch (every photon of every packed event in one
// simulate kernel, events kept apart by their genstep and photon ranges), runs up to `slots` such batches at once
// on separate CUDA streams so a new batch fills the SMs that the previous one's tail leaves idle, admits events
// only while the batch's device buffers fit the HBM budget, and hands back each event's hits in photon order with
// its submit-to-hits latency.  An event larger than a batch runs as genstep-aligned pieces in successive batches
// (the reference slices a large event the same way, qudarap/QSim.cc:481-529).  Each event's results are those it
// gets alone: its photons keep their event-local indices and the event's own Philox stream positions.

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <new>
#include <thread>
#include <unordered_map>

namespace {

using Clock = std::chrono::steady_clock;

// One piece's hits in host memory, left uninitialised until the device copy fills it
struct HitPiece {
    std::unique_ptr<gbo_sphoton[]> data;
    size_t n = 0;
};

struct ServerEvent {
    uint64_t ticket = 0;
    int32_t event_id = 0;
    std::vector<gbo_quad6> gs;
    std::vector<gbo_sphoton> input;
    long long num_photon = 0;
    Clock::time_point t_submit, t_done;
    int status = 0;             // 0 waiting, 1 on the GPU, 2 done, 3 failed
    std::string error;
    // an event larger than a batch runs as several pieces (genstep ranges), possibly in several slots at once
    int64_t next_gs = 0;                // first genstep not yet handed to a batch
    long long next_photon = 0;          // event-local index of that genstep's first photon
    int pieces_launched = 0, pieces_done = 0;
    bool all_launched = false;
    std::vector<HitPiece> piece_hits;   // hits of each piece, in photon order; the event's hits are their concatenation
    long long num_hit = 0;
};

// One batch entry: gensteps [g0, g1) of an event, whose photons are the event's [photon_offset, +num_photon)
struct Piece {
    std::shared_ptr<ServerEvent> ev;
    int64_t g0 = 0, g1 = 0;
    long long photon_offset = 0, num_photon = 0;
    int index = 0;
};

template <typename T>
struct HBuf {                   // pinned host staging
    T* ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t n)
    {
        if (n <= cap && ptr) return 0;
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
        size_t want = n < 1 ? 1 : n;
        if (cudaMallocHost(&ptr, want * sizeof(T)) != cudaSuccess) { ptr = nullptr; return fail(GBO_ERR_CUDA, "cudaMallocHost failed"); }
        cap = want;
        return 0;
    }
    void release() { if (ptr) cudaFreeHost(ptr); ptr = nullptr; cap = 0; }
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_kernels = nullptr, ev_done = nullptr;
    cudaGraphExec_t exec = nullptr;     // the slot's executable graph (graph mode)
    int phase = 0;              // 0 idle, 1 kernels running, 2 hit download running
    std::vector<Piece> pieces;
    long long num_photon = 0;
    bool big = false;           // holds a piece of at least target_batch_photon photons
    unsigned long long num_hit = 0;
    DBuf<gbo_quad6> gs;
    DBuf<unsigned long long> gs_end, ev_photon_begin, ev_pos0, ev_photon_offset, block_offset, counters, hit_gidx, ev_hit;
    DBuf<int> ev_gs_begin;
    DBuf<gbo_sphoton> input, hits_unordered, hits;
    DBuf<gbo_sphoton> gen_photon;       // kernel modes 2 and 3: the batch's pregenerated photons
    DBuf<ulonglong2> gen_rng;
    DBuf<int> gen_hint, gs_hint;        // start instance per pregenerated photon / per genstep
    WavefrontBufs wf;                   // kernel mode 3
    Wavefront wf_dev{};
    DBuf<uint32_t> bitmap, word_prefix, block_sum;
    HBuf<gbo_quad6> h_gs;
    HBuf<unsigned long long> h_gs_end, h_ev_photon_begin, h_ev_pos0, h_ev_photon_offset, h_ev_hit, h_counters;
    HBuf<int> h_ev_gs_begin;
    std::vector<HitPiece> staged;       // the current batch's hits per piece, copied from the device
    HBuf<gbo_sphoton> h_hits;           // pinned staging of a batch's hits when they are few
    bool direct = false;                // this batch's hits went straight into `staged`

    void release()
    {
        gs.release(); gs_end.release(); ev_photon_begin.release(); ev_pos0.release(); ev_photon_offset.release();
        block_offset.release(); counters.release(); hit_gidx.release(); ev_hit.release(); ev_gs_begin.release();
        input.release(); hits_unordered.release(); hits.release(); gen_photon.release(); gen_rng.release(); gen_hint.release(); gs_hint.release();
        wf.release();
        bitmap.release(); word_prefix.release();
        block_sum.release(); h_gs.release(); h_gs_end.release(); h_ev_photon_begin.release(); h_ev_pos0.release();
        h_ev_photon_offset.release(); h_ev_hit.release(); h_counters.release(); h_ev_gs_begin.release();
        staged.clear();
        h_hits.release();
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (ev_kernels) cudaEventDestroy(ev_kernels);
        if (ev_done) cudaEventDestroy(ev_done);
        if (stream) cudaStreamDestroy(stream);
        ev_kernels = ev_done = nullptr;
        stream = nullptr;
    }
};

// big batches in flight per GPU, over every server of the process (one server per geometry shares the GPU)
constexpr int SERVE_MAX_DEVICES = 64;
std::atomic<int> g_big_in_flight[SERVE_MAX_DEVICES];

std::atomic<int>& big_counter(int device) { return g_big_in_flight[device >= 0 && device < SERVE_MAX_DEVICES ? device : 0]; }

// a batch's hits above this size go straight from the device into per-piece host buffers
constexpr size_t SERVE_DIRECT_HIT_BYTES = 64ull << 20;

// device bytes per photon slot of a batch: bitmap + prefix bits, unordered + ordered hit capacity, hit index;
// kernel modes 2 and 3 add the pregenerated photon, its random-stream place and start instance; kernel mode 3 adds
// the hit record and five list entries (two step lists, the walk queue, its keys, the sorted queue)
constexpr double SERVE_BYTES_PER_PHOTON = 0.25 + 64.0 + 64.0 + 8.0;
constexpr double SERVE_BYTES_PER_PHOTON_GEN = 64.0 + 16.0 + 4.0;
constexpr double SERVE_BYTES_PER_PHOTON_WF = 32.0 + 20.0;

}  // namespace

struct gbo_server {
    gbo_engine* e = nullptr;
    gbo_server_config cfg{};
    long long max_batch_photon = 0;
    std::vector<Slot> slots;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<ServerEvent>> pending;
    std::unordered_map<uint64_t, std::shared_ptr<ServerEvent>> events;
    bool stop = false;
    uint64_t next_ticket = 1;
    gbo_server_stats stats{};
};

namespace {

// Every copy, memset and kernel of one batch, in stream order on the slot's stream (captured into a graph in
// graph mode): gensteps and entry tables up, the simulate launch, hit compaction, per-entry hit ranges and the
// counters back to pinned host memory.  Input photons are already on the device (copied before, see launch_batch).
int enqueue_batch(gbo_engine* e, Slot& sl, int n_ev, long long n_gs, bool has_input, long long N, long long words,
                  long long nblk)
{
    cudaStream_t s = sl.stream;
    if (n_gs) {
        CU(cudaMemcpyAsync(sl.gs.ptr, sl.h_gs.ptr, n_gs * sizeof(gbo_quad6), cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(sl.gs_end.ptr, sl.h_gs_end.ptr, n_gs * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
    }
    CU(cudaMemcpyAsync(sl.ev_gs_begin.ptr, sl.h_ev_gs_begin.ptr, (n_ev + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(sl.ev_photon_begin.ptr, sl.h_ev_photon_begin.ptr, (n_ev + 1) * sizeof(unsigned long long),
                       cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(sl.ev_pos0.ptr, sl.h_ev_pos0.ptr, n_ev * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(sl.ev_photon_offset.ptr, sl.h_ev_photon_offset.ptr, n_ev * sizeof(unsigned long long),
                       cudaMemcpyHostToDevice, s));
    CU(cudaMemsetAsync(sl.counters.ptr, 0, 4 * sizeof(unsigned long long), s));

    Params P = make_params(e);
    P.gs = reinterpret_cast<const float4*>(sl.gs.ptr);
    P.gs_end = sl.gs_end.ptr;
    P.num_gs = (int)n_gs;
    P.num_photon = N;
    P.input_photon = has_input ? sl.input.ptr : nullptr;
    P.hit_unordered = sl.hits_unordered.ptr;
    P.hit_count = sl.counters.ptr;
    P.bitmap = sl.bitmap.ptr;
    P.num_events = n_ev;
    P.ev_gs_begin = sl.ev_gs_begin.ptr;
    P.ev_photon_begin = sl.ev_photon_begin.ptr;
    P.ev_pos0 = sl.ev_pos0.ptr;
    P.ev_photon_offset = sl.ev_photon_offset.ptr;
    P.hit_gidx = sl.hit_gidx.ptr;
    if (e->cfg.kernel_mode >= 2) {
        P.gen_photon = sl.gen_photon.ptr;
        P.gen_rng = sl.gen_rng.ptr;
        P.gen_hint = sl.gen_hint.ptr;
    }
    if (N > 0) {
        if (e->cfg.kernel_mode != 1) CU(cudaMemsetAsync(sl.bitmap.ptr, 0, (size_t)words * sizeof(uint32_t), s));
        k_genstep_hint<<<(unsigned)((n_gs + 127) / 128), 128, 0, s>>>(P.acc, P.gs, (int)n_gs, sl.gs_hint.ptr);
        P.gs_hint = sl.gs_hint.ptr;
        launch_simulate(e, P, N, sl.counters.ptr + 2, s, nullptr, e->cfg.kernel_mode == 3 ? &sl.wf_dev : nullptr);
        CU(cudaGetLastError());
        k_word_prefix<<<(unsigned)nblk, SCAN_WORDS, 0, s>>>(sl.bitmap.ptr, words, sl.word_prefix.ptr, sl.block_sum.ptr);
        k_block_offsets<<<1, 1024, 0, s>>>(sl.block_sum.ptr, nblk, sl.block_offset.ptr, sl.counters.ptr + 1);
        k_gather_unordered<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(sl.hits_unordered.ptr, sl.counters.ptr, 0ull,
                                                                       sl.bitmap.ptr, sl.word_prefix.ptr,
                                                                       sl.block_offset.ptr, sl.hits.ptr, sl.hit_gidx.ptr);
        k_event_hit_ranges<<<(n_ev + 1 + 127) / 128, 128, 0, s>>>(sl.ev_photon_begin.ptr, n_ev, N, sl.bitmap.ptr,
                                                                  sl.word_prefix.ptr, sl.block_offset.ptr,
                                                                  sl.counters.ptr + 1, sl.ev_hit.ptr);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(sl.h_ev_hit.ptr, sl.ev_hit.ptr, (n_ev + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    } else {
        for (int k = 0; k <= n_ev; k++) sl.h_ev_hit.ptr[k] = 0;
    }
    CU(cudaMemcpyAsync(sl.h_counters.ptr, sl.counters.ptr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    return GBO_OK;
}

int launch_batch(gbo_server* sv, Slot& sl)
{
    gbo_engine* e = sv->e;
    cudaStream_t s = sl.stream;
    const int n_ev = (int)sl.pieces.size();
    long long n_gs = 0;
    bool has_input = false;
    for (const Piece& pc : sl.pieces) { n_gs += pc.g1 - pc.g0; has_input |= !pc.ev->input.empty(); }
    int rc;
    if ((rc = sl.h_gs.ensure(n_gs)) || (rc = sl.h_gs_end.ensure(n_gs)) || (rc = sl.h_ev_gs_begin.ensure(n_ev + 1)) ||
        (rc = sl.h_ev_photon_begin.ensure(n_ev + 1)) || (rc = sl.h_ev_pos0.ensure(n_ev)) ||
        (rc = sl.h_ev_photon_offset.ensure(n_ev)) || (rc = sl.h_ev_hit.ensure(n_ev + 1)) || (rc = sl.h_counters.ensure(4)))
        return rc;
    long long g = 0;
    unsigned long long total = 0;
    for (int k = 0; k < n_ev; k++) {
        const Piece& pc = sl.pieces[k];
        const ServerEvent& ev = *pc.ev;
        sl.h_ev_gs_begin.ptr[k] = (int)g;
        sl.h_ev_photon_begin.ptr[k] = total;
        sl.h_ev_pos0.ptr[k] = e->cfg.rng_offset + e->cfg.event_skipahead * (uint64_t)(ev.event_id < 0 ? 0 : ev.event_id);
        sl.h_ev_photon_offset.ptr[k] = (unsigned long long)pc.photon_offset;
        for (int64_t i = pc.g0; i < pc.g1; i++) {
            const gbo_quad6& q = ev.gs[(size_t)i];
            sl.h_gs.ptr[g] = q;
            total += q.q[0].u[3];
            sl.h_gs_end.ptr[g] = total;
            g++;
        }
    }
    sl.h_ev_gs_begin.ptr[n_ev] = (int)g;
    sl.h_ev_photon_begin.ptr[n_ev] = total;
    const long long N = (long long)total;
    sl.num_photon = N;
    const long long words = (N + 31) / 32;
    const long long nblk = (words + SCAN_WORDS - 1) / SCAN_WORDS;
    if ((rc = sl.gs.ensure(n_gs)) || (rc = sl.gs_end.ensure(n_gs)) || (rc = sl.ev_gs_begin.ensure(n_ev + 1)) ||
        (rc = sl.ev_photon_begin.ensure(n_ev + 1)) || (rc = sl.ev_pos0.ensure(n_ev)) ||
        (rc = sl.ev_photon_offset.ensure(n_ev)) || (rc = sl.ev_hit.ensure(n_ev + 1)) ||
        (rc = sl.counters.ensure(4)) || (rc = sl.bitmap.ensure(words)) || (rc = sl.word_prefix.ensure(words)) ||
        (rc = sl.block_sum.ensure(nblk)) || (rc = sl.block_offset.ensure(nblk)) || (rc = sl.hits_unordered.ensure(N)) ||
        (rc = sl.hit_gidx.ensure(N)) || (rc = sl.hits.ensure(N)) || (has_input && (rc = sl.input.ensure(N))) ||
        (rc = sl.gs_hint.ensure(n_gs > 0 ? n_gs : 1)) ||
        (e->cfg.kernel_mode >= 2 &&
         ((rc = sl.gen_photon.ensure(N)) || (rc = sl.gen_rng.ensure(N)) || (rc = sl.gen_hint.ensure(N)))) ||
        (e->cfg.kernel_mode == 3 && (rc = sl.wf.ensure(N, e->cfg.max_bounce, e->cfg.precision != 0, sl.wf_dev))))
        return rc;
    // input photons go up straight from each event's own copy, one copy per piece at the piece's launch position
    // (outside any graph: the source is pageable host memory)
    if (has_input) {
        for (int k = 0; k < n_ev; k++) {
            const Piece& pc = sl.pieces[k];
            const std::vector<gbo_sphoton>& in = pc.ev->input;
            const long long avail = (long long)in.size() - pc.photon_offset;
            const long long n = avail < pc.num_photon ? avail : pc.num_photon;
            if (n > 0)
                CU(cudaMemcpyAsync(sl.input.ptr + sl.h_ev_photon_begin.ptr[k], in.data() + pc.photon_offset,
                                   (size_t)n * sizeof(gbo_sphoton), cudaMemcpyHostToDevice, s));
        }
    }
    int rc2 = GBO_OK;
    if (!sv->cfg.use_graph) {
        rc2 = enqueue_batch(e, sl, n_ev, n_gs, has_input, N, words, nblk);
    } else {
        // capture the batch into a graph, then update the slot's executable graph in place (kernel arguments,
        // grid sizes and copy sizes change from batch to batch; the topology changes only with input photons or
        // an empty batch, and then the graph is instantiated afresh)
        CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        rc2 = enqueue_batch(e, sl, n_ev, n_gs, has_input, N, words, nblk);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (!rc2 && ce != cudaSuccess) rc2 = fail(GBO_ERR_CUDA, "batch capture failed: %s", cudaGetErrorString(ce));
        if (!rc2 && sl.exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(sl.exec, graph, &info) != cudaSuccess) {
                (void)cudaGetLastError();
                cudaGraphExecDestroy(sl.exec);
                sl.exec = nullptr;
            }
        }
        if (!rc2 && !sl.exec) {
            const cudaError_t ie = cudaGraphInstantiate(&sl.exec, graph, 0);
            if (ie != cudaSuccess) { sl.exec = nullptr; rc2 = fail(GBO_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ie)); }
            else sv->stats.graph_instantiations++;
        }
        if (graph) cudaGraphDestroy(graph);
        if (!rc2) {
            const cudaError_t le = cudaGraphLaunch(sl.exec, s);
            if (le != cudaSuccess) rc2 = fail(GBO_ERR_CUDA, "graph launch failed: %s", cudaGetErrorString(le));
            else sv->stats.graph_launches++;
        }
    }
    if (rc2) return rc2;
    CU(cudaEventRecord(sl.ev_kernels, s));
    sl.phase = 1;
    return GBO_OK;
}

void finish_slot(gbo_server* sv, Slot& sl, int rc)
{
    std::lock_guard<std::mutex> lock(sv->mu);
    const Clock::time_point now = Clock::now();
    for (size_t k = 0; k < sl.pieces.size(); k++) {
        const Piece& pc = sl.pieces[k];
        ServerEvent& ev = *pc.ev;
        ev.pieces_done++;
        if (ev.status == 3) continue;                   // an earlier piece failed
        if (rc != GBO_OK) {
            ev.status = 3;
            ev.error = g_last_error;
            ev.t_done = now;
            sv->stats.events_done++;
            continue;
        }
        if (!sl.direct) {                               // split the pinned staging into the pieces
            const unsigned long long a = sl.h_ev_hit.ptr[k], n = sl.h_ev_hit.ptr[k + 1] - a;
            sl.staged[k].n = (size_t)n;
            if (n) {
                sl.staged[k].data.reset(new (std::nothrow) gbo_sphoton[n]);
                if (!sl.staged[k].data) {
                    ev.status = 3;
                    ev.error = "host memory for hits";
                    ev.t_done = now;
                    sv->stats.events_done++;
                    continue;
                }
                std::memcpy(sl.staged[k].data.get(), sl.h_hits.ptr + a, (size_t)n * sizeof(gbo_sphoton));
            }
        }
        if ((int)ev.piece_hits.size() <= pc.index) ev.piece_hits.resize((size_t)pc.index + 1);
        ev.num_hit += (long long)sl.staged[k].n;
        ev.piece_hits[(size_t)pc.index] = std::move(sl.staged[k]);
        if (ev.all_launched && ev.pieces_done == ev.pieces_launched) {
            ev.status = 2;
            ev.t_done = now;
            sv->stats.events_done++;
        }
    }
    sv->stats.batches++;
    sv->stats.photons += sl.num_photon;
    if (sl.big) big_counter(sv->e->device)--;
    sl.big = false;
    sl.pieces.clear();
    sl.phase = 0;
    sv->cv_done.notify_all();
}

void serve_loop(gbo_server* sv)
{
    cudaSetDevice(sv->e->device);
    for (;;) {
        bool busy = false;
        for (Slot& sl : sv->slots) {
            if (sl.phase == 1) {
                busy = true;
                cudaError_t q = cudaEventQuery(sl.ev_kernels);
                if (q == cudaErrorNotReady) continue;
                if (q != cudaSuccess) { fail(GBO_ERR_CUDA, "batch failed: %s", cudaGetErrorString(q)); finish_slot(sv, sl, GBO_ERR_CUDA); continue; }
                sl.num_hit = sl.h_counters.ptr[1];
                // few hits: one asynchronous copy into pinned staging, split per piece when the batch finishes;
                // many hits: each piece's hits straight into host memory of its own (no second copy, no zero fill)
                int rc = GBO_OK;
                sl.staged.clear();
                sl.staged.resize(sl.pieces.size());
                sl.direct = sl.num_hit * sizeof(gbo_sphoton) > SERVE_DIRECT_HIT_BYTES;
                if (!sl.direct) {
                    rc = sl.h_hits.ensure(sl.num_hit);
                    if (!rc && sl.num_hit &&
                        cudaMemcpyAsync(sl.h_hits.ptr, sl.hits.ptr, sl.num_hit * sizeof(gbo_sphoton), cudaMemcpyDeviceToHost,
                                        sl.stream) != cudaSuccess)
                        rc = fail(GBO_ERR_CUDA, "hit download failed");
                }
                for (size_t k = 0; k < sl.pieces.size() && !rc && sl.direct; k++) {
                    const unsigned long long a = sl.h_ev_hit.ptr[k], n = sl.h_ev_hit.ptr[k + 1] - a;
                    sl.staged[k].n = (size_t)n;
                    if (!n) continue;
                    sl.staged[k].data.reset(new (std::nothrow) gbo_sphoton[n]);
                    if (!sl.staged[k].data) { rc = fail(GBO_ERR_CAPACITY, "host memory for %llu hits", n); break; }
                    if (cudaMemcpyAsync(sl.staged[k].data.get(), sl.hits.ptr + a, (size_t)n * sizeof(gbo_sphoton),
                                        cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
                        rc = fail(GBO_ERR_CUDA, "hit download failed");
                }
                if (!rc && cudaEventRecord(sl.ev_done, sl.stream) != cudaSuccess) rc = fail(GBO_ERR_CUDA, "event record failed");
                if (rc) { finish_slot(sv, sl, rc); continue; }
                // the batch's kernels are done: a waiting big event may start in another slot while these hits
                // download, so the GPU does not idle through the copy
                if (sl.big) { big_counter(sv->e->device)--; sl.big = false; }
                sl.phase = 2;
            } else if (sl.phase == 2) {
                busy = true;
                cudaError_t q = cudaEventQuery(sl.ev_done);
                if (q == cudaErrorNotReady) continue;
                finish_slot(sv, sl, q == cudaSuccess ? GBO_OK : fail(GBO_ERR_CUDA, "hit download: %s", cudaGetErrorString(q)));
            }
        }
        // admit waiting events into idle slots: at once when the GPU has nothing in flight, otherwise only once
        // enough photons wait to fill the GPU (min_batch_photon), so that batches do not degenerate to single events.
        // A big event (at least target_batch_photon photons, enough to fill the GPU alone) never starts beside
        // another big one's kernels, where the two would share the SMs and each take twice as long (it may start
        // while the other's hits download), and never joins a batch of small events, whose latency would become its
        // own; small events may pass a waiting big one into the free slot unless big_exclusive keeps the GPU for
        // the big one's kernels.
        for (Slot& sl : sv->slots) {
            if (sl.phase != 0) continue;
            int in_flight = 0;
            bool big_in_flight = false;
            for (Slot& x : sv->slots) in_flight += x.phase != 0;
            big_in_flight = big_counter(sv->e->device).load() > 0;
            if (big_in_flight && sv->cfg.big_exclusive) continue;
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                auto admissible = [&](const ServerEvent& ev) {
                    return !big_in_flight || ev.num_photon - ev.next_photon < sv->cfg.target_batch_photon;
                };
                if (in_flight > 0) {
                    // small events wait for company while the GPU is busy, but not longer than max_wait_us: a chain
                    // of big launches would otherwise hold them until it ends
                    long long waiting = 0;
                    Clock::time_point oldest = Clock::time_point::max();
                    for (auto& ev : sv->pending) {
                        if (!admissible(*ev)) continue;
                        waiting += ev->num_photon - ev->next_photon;
                        if (ev->t_submit < oldest) oldest = ev->t_submit;
                        if (waiting >= sv->cfg.min_batch_photon) break;
                    }
                    const bool overdue = waiting > 0 && sv->cfg.max_wait_us > 0 &&
                                         Clock::now() - oldest >= std::chrono::microseconds(sv->cfg.max_wait_us);
                    if (waiting < sv->cfg.min_batch_photon && !overdue) continue;
                }
                long long photons = 0;
                sl.big = false;
                for (auto it = sv->pending.begin(); it != sv->pending.end();) {
                    std::shared_ptr<ServerEvent> ev = *it;
                    const long long rest = ev->num_photon - ev->next_photon;
                    if (!admissible(*ev)) { ++it; continue; }
                    if (!sl.pieces.empty() && rest >= sv->cfg.target_batch_photon) { ++it; continue; }
                    if (!sl.pieces.empty() && (photons + rest > sv->max_batch_photon ||
                                               photons >= sv->cfg.target_batch_photon ||
                                               (int)sl.pieces.size() >= sv->cfg.max_batch_events))
                        break;
                    // the rest of the event, or, when it does not fit an empty batch, its next genstep-aligned piece
                    // of at most max_batch_photon photons (a single larger genstep goes alone)
                    Piece pc;
                    pc.ev = ev;
                    pc.g0 = ev->next_gs;
                    pc.photon_offset = ev->next_photon;
                    int64_t g1 = pc.g0;
                    long long n = 0;
                    const int64_t ng = (int64_t)ev->gs.size();
                    while (g1 < ng && (g1 == pc.g0 || n + (long long)ev->gs[(size_t)g1].q[0].u[3] <= sv->max_batch_photon - photons))
                        n += ev->gs[(size_t)g1++].q[0].u[3];
                    pc.g1 = g1;
                    pc.num_photon = n;
                    pc.index = ev->pieces_launched++;
                    ev->next_gs = g1;
                    ev->next_photon += n;
                    ev->status = 1;
                    photons += n;
                    sl.big |= n >= sv->cfg.target_batch_photon;
                    sl.pieces.push_back(pc);
                    if (g1 < ng) break;                 // the event goes on in a later batch
                    ev->all_launched = true;
                    it = sv->pending.erase(it);
                }
            }
            if (sl.pieces.empty()) continue;
            if (sl.big) big_counter(sv->e->device)++;
            busy = true;
            int rc = launch_batch(sv, sl);
            if (rc) finish_slot(sv, sl, rc);
        }
        std::unique_lock<std::mutex> lock(sv->mu);
        if (sv->stop && sv->pending.empty()) {
            bool idle = true;
            for (Slot& sl : sv->slots) idle = idle && sl.phase == 0;
            if (idle) break;
        }
        if (busy) {
            lock.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        } else {
            sv->cv_work.wait_for(lock, std::chrono::milliseconds(2));
        }
    }
}

}  // namespace

extern "C" {

int gbo_server_config_default(gbo_server_config* c)
{
    if (!c) return fail(GBO_ERR_ARG, "gbo_server_config_default: null config");
    std::memset(c, 0, sizeof(*c));
    c->slots = 2;
    c->max_batch_photon = 64ll << 20;
    c->hbm_budget_bytes = 120ll << 30;
    c->max_batch_events = 4096;
    c->min_batch_photon = 2ll << 20;
    c->use_graph = 1;
    c->target_batch_photon = 4ll << 20;
    c->max_wait_us = 1000;
    return GBO_OK;
}

int gbo_server_create(gbo_engine* e, const gbo_server_config* cfg, gbo_server** out)
{
    if (!e || !out) return fail(GBO_ERR_ARG, "gbo_server_create: null argument");
    *out = nullptr;
    gbo_server_config c;
    if (cfg) c = *cfg; else gbo_server_config_default(&c);
    if (c.slots < 1 || c.slots > 8) return fail(GBO_ERR_ARG, "gbo_server_create: slots %d not in 1..8", c.slots);
    if (c.max_batch_events < 1) return fail(GBO_ERR_ARG, "gbo_server_create: max_batch_events must be positive");
    if (c.target_batch_photon <= 0) c.target_batch_photon = INT64_MAX;     // no target: max_batch_photon alone
    CU(cudaSetDevice(e->device));
    auto* sv = new gbo_server();
    sv->e = e;
    sv->cfg = c;
    const double per_photon = SERVE_BYTES_PER_PHOTON + (e->cfg.kernel_mode >= 2 ? SERVE_BYTES_PER_PHOTON_GEN : 0.0) +
                              (e->cfg.kernel_mode == 3 ? SERVE_BYTES_PER_PHOTON_WF : 0.0) +
                              (e->cfg.kernel_mode == 3 && e->cfg.precision ? (double)sizeof(Acc64) : 0.0);
    const long long by_budget = (long long)((double)c.hbm_budget_bytes / (per_photon * c.slots));
    sv->max_batch_photon = c.max_batch_photon > 0 && c.max_batch_photon < by_budget ? c.max_batch_photon : by_budget;
    if (sv->max_batch_photon < 1) { delete sv; return fail(GBO_ERR_CAPACITY, "gbo_server_create: HBM budget below one photon per slot"); }
    sv->slots.resize((size_t)c.slots);
    for (Slot& sl : sv->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev_kernels, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev_done, cudaEventDisableTiming) != cudaSuccess) {
            for (Slot& x : sv->slots) x.release();
            delete sv;
            return fail(GBO_ERR_CUDA, "gbo_server_create: stream/event creation failed");
        }
    }
    sv->worker = std::thread(serve_loop, sv);
    *out = sv;
    return GBO_OK;
}

int gbo_server_submit(gbo_server* sv, int32_t event_id, const gbo_quad6* gs, int64_t num_gs, const gbo_sphoton* input_photon,
                      int64_t num_input_photon, uint64_t* ticket)
{
    if (!sv || !ticket) return fail(GBO_ERR_ARG, "gbo_server_submit: null argument");
    if (num_gs < 0 || (num_gs > 0 && !gs)) return fail(GBO_ERR_ARG, "gbo_server_submit: bad gensteps");
    if (num_input_photon < 0 || (num_input_photon > 0 && !input_photon)) return fail(GBO_ERR_ARG, "gbo_server_submit: bad input photons");
    auto ev = std::make_shared<ServerEvent>();
    ev->event_id = event_id;
    ev->gs.assign(gs, gs + num_gs);
    if (num_input_photon) ev->input.assign(input_photon, input_photon + num_input_photon);
    long long n = 0;
    bool has_input_gs = false;
    for (const gbo_quad6& q : ev->gs) { n += q.q[0].u[3]; has_input_gs |= q.q[0].i[0] == GBO_GS_INPUT_PHOTON; }
    if (has_input_gs && num_input_photon < n)
        return fail(GBO_ERR_ARG, "gbo_server_submit: INPUT_PHOTON gensteps need %lld photons, %lld given", n, (long long)num_input_photon);
    ev->num_photon = n;
    ev->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (sv->stop) return fail(GBO_ERR_STATE, "gbo_server_submit: server stopping");
        ev->ticket = sv->next_ticket++;
        sv->events[ev->ticket] = ev;
        sv->pending.push_back(ev);
        sv->stats.events_submitted++;
    }
    sv->cv_work.notify_one();
    *ticket = ev->ticket;
    return GBO_OK;
}

int gbo_server_wait(gbo_server* sv, uint64_t ticket, int64_t timeout_us)
{
    if (!sv) return fail(GBO_ERR_ARG, "gbo_server_wait: null server");
    std::unique_lock<std::mutex> lock(sv->mu);
    auto it = sv->events.find(ticket);
    if (it == sv->events.end()) return fail(GBO_ERR_ARG, "gbo_server_wait: unknown ticket %llu", (unsigned long long)ticket);
    std::shared_ptr<ServerEvent> ev = it->second;
    auto done = [&] { return ev->status >= 2; };
    if (timeout_us < 0 || timeout_us > (1ll << 40)) sv->cv_done.wait(lock, done);      // beyond ~12 days: no limit
    else if (!sv->cv_done.wait_for(lock, std::chrono::microseconds(timeout_us), done))
        return fail(GBO_ERR_TIMEOUT, "gbo_server_wait: event %llu not done", (unsigned long long)ticket);
    if (ev->status == 3) return fail(GBO_ERR_DEVICE, "event %llu failed: %s", (unsigned long long)ticket, ev->error.c_str());
    return GBO_OK;
}

int gbo_server_event_info(gbo_server* sv, uint64_t ticket, int64_t* num_photon, int64_t* num_hit, double* latency_s)
{
    if (!sv) return fail(GBO_ERR_ARG, "gbo_server_event_info: null server");
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->events.find(ticket);
    if (it == sv->events.end()) return fail(GBO_ERR_ARG, "gbo_server_event_info: unknown ticket");
    ServerEvent& ev = *it->second;
    if (ev.status < 2) return fail(GBO_ERR_STATE, "gbo_server_event_info: event not done");
    if (num_photon) *num_photon = ev.num_photon;
    if (num_hit) *num_hit = (int64_t)ev.num_hit;
    if (latency_s) *latency_s = std::chrono::duration<double>(ev.t_done - ev.t_submit).count();
    return GBO_OK;
}

int gbo_server_copy_hits(gbo_server* sv, uint64_t ticket, gbo_sphoton* dst, int64_t offset, int64_t count)
{
    if (!sv || (!dst && count > 0)) return fail(GBO_ERR_ARG, "gbo_server_copy_hits: null argument");
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->events.find(ticket);
    if (it == sv->events.end()) return fail(GBO_ERR_ARG, "gbo_server_copy_hits: unknown ticket");
    ServerEvent& ev = *it->second;
    if (ev.status != 2) return fail(GBO_ERR_STATE, "gbo_server_copy_hits: event not done");
    if (offset < 0 || count < 0 || offset + count > (int64_t)ev.num_hit) return fail(GBO_ERR_ARG, "gbo_server_copy_hits: range outside hits");
    int64_t base = 0;                                   // concatenation of the pieces, in piece order
    for (const HitPiece& pc : ev.piece_hits) {
        const int64_t n = (int64_t)pc.n;
        const int64_t lo = offset > base ? offset : base, hi = offset + count < base + n ? offset + count : base + n;
        if (hi > lo) std::memcpy(dst + (lo - offset), pc.data.get() + (lo - base), (size_t)(hi - lo) * sizeof(gbo_sphoton));
        base += n;
    }
    return GBO_OK;
}

int gbo_server_release(gbo_server* sv, uint64_t ticket)
{
    if (!sv) return fail(GBO_ERR_ARG, "gbo_server_release: null server");
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->events.find(ticket);
    if (it == sv->events.end()) return fail(GBO_ERR_ARG, "gbo_server_release: unknown ticket");
    if (it->second->status < 2) return fail(GBO_ERR_STATE, "gbo_server_release: event still in flight");
    sv->events.erase(it);
    return GBO_OK;
}

int gbo_server_get_stats(gbo_server* sv, gbo_server_stats* out)
{
    if (!sv || !out) return fail(GBO_ERR_ARG, "gbo_server_get_stats: null argument");
    std::lock_guard<std::mutex> lock(sv->mu);
    *out = sv->stats;
    out->max_batch_photon = sv->max_batch_photon;
    return GBO_OK;
}

void gbo_server_destroy(gbo_server* sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    cudaSetDevice(sv->e->device);
    for (Slot& sl : sv->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        sl.release();
    }
    delete sv;
}

// ---- event API on the engine handle ----------------------------------------------------------------------------

static gbo_server* engine_event_server(gbo_engine* e)
{
    std::lock_guard<std::mutex> lock(e->event_server_mu);
    if (!e->event_server) {
        gbo_server_config c;
        gbo_server_config_default(&c);
        if (gbo_server_create(e, &c, &e->event_server) != GBO_OK) e->event_server = nullptr;
    }
    return e->event_server;
}

int gbo_event_submit_photons(gbo_engine* e, const gbo_quad6* gs, size_t num_gs, const gbo_sphoton* input_photon,
                             size_t num_input_photon, uint32_t event_id, gbo_ticket* ticket)
{
    if (!e || !ticket) return fail(GBO_ERR_ARG, "gbo_event_submit: null argument");
    if (event_id > 0x7fffffffu) return fail(GBO_ERR_ARG, "gbo_event_submit: event id %u above 2^31-1", event_id);
    gbo_server* sv = engine_event_server(e);
    if (!sv) return GBO_ERR_CUDA;                       // gbo_server_create recorded the reason
    return gbo_server_submit(sv, (int32_t)event_id, gs, (int64_t)num_gs, input_photon, (int64_t)num_input_photon,
                             ticket);
}

int gbo_event_submit(gbo_engine* e, const gbo_quad6* gs, size_t num_gs, uint32_t event_id, gbo_ticket* ticket)
{
    return gbo_event_submit_photons(e, gs, num_gs, nullptr, 0, event_id, ticket);
}

static gbo_server* engine_server_of(gbo_engine* e, const char* what)
{
    if (!e) { fail(GBO_ERR_ARG, "%s: null engine", what); return nullptr; }
    std::lock_guard<std::mutex> lock(e->event_server_mu);
    if (!e->event_server) fail(GBO_ERR_STATE, "%s: no event submitted", what);
    return e->event_server;
}

int gbo_event_wait(gbo_engine* e, gbo_ticket ticket, int64_t timeout_ns)
{
    gbo_server* sv = engine_server_of(e, "gbo_event_wait");
    if (!sv) return e ? GBO_ERR_STATE : GBO_ERR_ARG;
    // round up so that a positive timeout never becomes a zero one
    const int64_t us = timeout_ns < 0 ? -1 : timeout_ns / 1000 + (timeout_ns % 1000 != 0 ? 1 : 0);
    return gbo_server_wait(sv, ticket, us);
}

int64_t gbo_event_num_hits(gbo_engine* e, gbo_ticket ticket)
{
    gbo_server* sv = engine_server_of(e, "gbo_event_num_hits");
    if (!sv) return -(int64_t)(e ? GBO_ERR_STATE : GBO_ERR_ARG);
    int64_t n = 0;
    const int rc = gbo_server_event_info(sv, ticket, nullptr, &n, nullptr);
    return rc == GBO_OK ? n : -(int64_t)rc;
}

int gbo_event_copy_hits(gbo_engine* e, gbo_ticket ticket, gbo_sphoton* dst, size_t n)
{
    gbo_server* sv = engine_server_of(e, "gbo_event_copy_hits");
    if (!sv) return e ? GBO_ERR_STATE : GBO_ERR_ARG;
    return gbo_server_copy_hits(sv, ticket, dst, 0, (int64_t)n);
}

int gbo_event_release(gbo_engine* e, gbo_ticket ticket)
{
    gbo_server* sv = engine_server_of(e, "gbo_event_release");
    if (!sv) return e ? GBO_ERR_STATE : GBO_ERR_ARG;
    return gbo_server_release(sv, ticket);
}

int gbo_geometry_create(const gbo_geometry_desc* g, gbo_geometry** out)
{
    gbo_config c;
    gbo_config_default(&c);
    return gbo_engine_create(g, &c, 0, out);
}

void gbo_geometry_destroy(gbo_geometry* g) { gbo_engine_destroy(g); }

}  // extern "C"
