// server.cu -- continuous-batching request server (include/erlbm_gb300.h, erlbm_server_*).
//
// The reference has no serving path; this is the device-resident request loop that admits
// independent runs of mixed sizes while others are on the GPU.  Two lanes:
//
//  slot lane    D3Q19 lattices of <= 288 nodes (Taylor-Green map points, the obstacle channel at
//               scale 1).  A persistent kernel per precision (k_slot_server) stays resident; its CTAs
//               claim requests from a ring in mapped pinned memory as soon as the host publishes
//               them, run each to completion in shared memory and publish the result.  Idle CTAs
//               poll with a bounded wait and exit; the scheduler relaunches the loop on demand.
//  team lane    D2Q9 Taylor-Green up to 512^2, D3Q19 Taylor-Green up to 64^3, the obstacle channel
//               scaled by more than 1 (team_lane.cuh).  A second persistent kernel per precision:
//               its admitter claims requests from another ring and admits them on the device by
//               HBM footprint (pages of the team arena); its CTAs join the admitted runs and work
//               through their items (chunks of nodes per step), and publish the results.  No host
//               launch per run or per step.
//  stream lane  every larger lattice.  Each admitted run gets device memory from a fixed HBM arena
//               (admission is by footprint: a request waits until its populations, scratch and
//               status fit), its own non-blocking CUDA stream, and is advanced in chunks of steps;
//               runs on different streams overlap on the device.
//
// One scheduler thread issues every CUDA call (no allocation or device-wide synchronisation after
// start-up, so nothing ever waits for the resident loops).  Results are deterministic: the lane a
// request takes depends only on the request and the server's configuration, and the team and stream
// lanes give the same bits, so a run gives the same result alone and in a mix.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/erlbm_gb300.h"
#include "abi_internal.h"
#include "batch_kernels.cuh"
#include "kernels_api.h"
#include "team_lane.cuh"

using namespace erlbm;

namespace {

using Clock = std::chrono::steady_clock;

// First-fit sub-allocator over one cudaMalloc'd block (the server's HBM budget).
class Arena {
public:
    int init(size_t bytes)
    {
        size_ = bytes;
        cudaError_t e = cudaMalloc(&base_, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "server arena");
        free_[0] = bytes;
        return ERLBM_OK;
    }
    ~Arena()
    {
        if (base_) cudaFree(base_);
    }
    void *alloc(size_t bytes)
    {
        bytes = (bytes + 255) / 256 * 256;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const size_t off = it->first, rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                used_ += bytes;
                sizes_[off] = bytes;
                return (char *)base_ + off;
            }
        }
        return nullptr;
    }
    void release(void *p)
    {
        if (!p) return;
        const size_t off = (char *)p - (char *)base_;
        auto s = sizes_.find(off);
        if (s == sizes_.end()) return;
        size_t size = s->second;
        sizes_.erase(s);
        used_ -= size;
        size_t o = off;
        auto next = free_.lower_bound(o);
        if (next != free_.end() && next->first == o + size) {
            size += next->second;
            free_.erase(next);
        }
        auto it = free_.lower_bound(o);
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == o) {
                o = prev->first;
                size += prev->second;
                free_.erase(prev);
            }
        }
        free_[o] = size;
    }
    size_t used() const { return used_; }
    size_t size() const { return size_; }

private:
    void *base_ = nullptr;
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
    std::map<size_t, size_t> sizes_;
};

constexpr int MAX_SLOT_NODES = 288;

struct SlotLane {
    int prec = 0;
    SlotEntry *h_entries = nullptr;
    SlotDone *h_done = nullptr;
    int *h_tail = nullptr;  // [0] tail, [1] stop
    int *d_head = nullptr, *d_exits = nullptr;
    BatchGeo *d_geos = nullptr;
    SlotRing ring{};
    cudaStream_t stream = nullptr;
    cudaEvent_t exited = nullptr;
    bool running = false;
    int published = 0;
    int grid = 0, block = 0;
    size_t smem = 0;
    std::unordered_map<int, int64_t> ticket_of;  // ring index -> ticket
    std::vector<int> outstanding;
};

// A stream of the stream lane with its pinned result words and completion event.
struct StreamSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    double *h_out = nullptr;  // pinned: [0] energy, [2..3] RunStatus
};

// The team lane of one precision: its ring of requests and results in mapped pinned memory and the
// device state of its resident launch.
struct TeamLane {
    int prec = 0;
    TeamEntry *h_entries = nullptr;
    unsigned char *h_payload = nullptr;  // mapped: TEAM_PAYLOAD bytes per ring entry
    TeamDone *h_done = nullptr;
    int *h_tail = nullptr;  // [0] tail, [1] stop
    TeamRing ring{};
    TeamCtl *d_ctl = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t exited = nullptr;
    bool running = false;
    int published = 0, grid = 0;
    std::unordered_map<int, int64_t> ticket_of;  // ring index -> ticket
    std::vector<int> outstanding;
};

constexpr int TEAM_CAPACITY = 128;            // ring entries per team lane
constexpr long long TEAM_PAYLOAD = 64 << 10;  // payload bytes per ring entry

struct Job {
    int64_t ticket = 0;
    StreamSlot *slot = nullptr;
    erlbm_request req{};
    int q = 0, prec = 0;
    Geo g{};
    BCp bc{};
    Relax R{};
    long long n_fluid = 0;
    void *buf[2] = {nullptr, nullptr};
    int cur = 0, kind = 0;
    double *scr = nullptr;   // n_fluid + 4096 doubles
    RunStatus *status = nullptr;
    uint8_t *solid = nullptr;
    int *nof = nullptr;
    double *tab = nullptr;
    double *h_out = nullptr;  // pinned: [0] energy, [1..2] status bits
    long long steps_done = 0;
    bool check_density = false;
    bool finalizing = false;
    bool in_flight = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<void *> mem;
    double t_admit = 0;
};

// A stream-lane request waiting for admission, with its submission time and estimated GPU time.
struct Pending {
    int64_t ticket = 0;
    erlbm_request req{};
    double t_submit = 0;
    double est = 0;  // seconds
};

}  // namespace

struct erlbm_server {
    erlbm_server_desc desc{};
    int device = 0, sms = 1;
    Clock::time_point t0;
    Arena arena;
    SlotLane lane[2];
    TeamLane team[2];             // [0] FP64, [1] FP32-shifted
    char *team_arena = nullptr;   // pages of the team lanes
    unsigned *d_pages = nullptr;  // their bitmap
    int team_pages = 0;
    double team_clock = 0;        // server clock minus the device clock (s)
    int team_jobs = TEAM_MAX_JOBS;  // runs admitted at a time per team loop
    std::deque<std::pair<int64_t, erlbm_request>> pending_c[2];  // team-lane requests waiting for ring space
    BatchGeo geos_host[2]{};
    uint8_t *d_obst_solid = nullptr;
    double *d_tg_tab = nullptr;
    std::vector<StreamSlot *> streams;     // free stream slots
    std::vector<StreamSlot *> all_streams;
    std::vector<Job *> active;
    std::deque<std::pair<int64_t, erlbm_request>> pending_a[2];  // slot-lane requests waiting for ring space
    std::vector<Pending> pending_b;  // stream-lane requests waiting for memory and a stream
    // submission and results (shared with user threads)
    std::mutex mu;
    std::condition_variable cv_done, cv_work;
    std::deque<std::pair<int64_t, erlbm_request>> inbox;
    std::unordered_map<int64_t, erlbm_result> results;
    std::unordered_map<int64_t, double> t_submit;
    int64_t next_ticket = 1;
    std::atomic<bool> stopping{false};
    std::thread th;
    int fatal = 0;
    std::string fatal_msg;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

bool slot_eligible(const erlbm_request &r)
{
    if (r.kind == ERLBM_REQ_TG_MAP_POINT) return r.L == 16 || r.L == 0;
    if (r.kind == ERLBM_REQ_OBSTACLE) return r.sx <= 1 && r.sy <= 1;
    return false;
}

void finish(erlbm_server *s, int64_t ticket, erlbm_result r)
{
    std::lock_guard<std::mutex> lk(s->mu);
    r.t_submit = s->t_submit[ticket];
    r.t_done = s->now();
    s->results[ticket] = r;
    s->cv_done.notify_all();
}

erlbm_result error_result(int code, int lane)
{
    erlbm_result r;
    memset(&r, 0, sizeof(r));
    r.status = code;
    r.lane = lane;
    return r;
}

// ---- slot lane --------------------------------------------------------------------------------

int lane_setup(erlbm_server *s, SlotLane &L, int prec)
{
    L.prec = prec;
    const int cap = s->desc.queue_capacity;
    cudaError_t e;
    if ((e = cudaHostAlloc(&L.h_entries, (size_t)cap * sizeof(SlotEntry), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc(&L.h_done, (size_t)cap * sizeof(SlotDone), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc(&L.h_tail, 64, cudaHostAllocMapped)) != cudaSuccess)
        return cuda_fail(e, "server ring");
    memset(L.h_done, 0, (size_t)cap * sizeof(SlotDone));
    memset(L.h_tail, 0, 64);
    L.d_head = (int *)s->arena.alloc(64);
    L.d_exits = L.d_head + 4;
    L.d_geos = (BatchGeo *)s->arena.alloc(2 * sizeof(BatchGeo));
    if (!L.d_head || !L.d_geos) {
        set_error("server arena too small for the slot lane%s%s", "", "");
        return ERLBM_E_OOM;
    }
    if ((e = cudaMemset(L.d_head, 0, 64)) != cudaSuccess) return cuda_fail(e, "server ring");
    if ((e = cudaMemcpy(L.d_geos, s->geos_host, 2 * sizeof(BatchGeo), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "server geometries");
    SlotEntry *de;
    SlotDone *dd;
    int *dt;
    if ((e = cudaHostGetDevicePointer(&de, L.h_entries, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&dd, L.h_done, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&dt, L.h_tail, 0)) != cudaSuccess)
        return cuda_fail(e, "server ring mapping");
    L.ring.tail = dt;
    L.ring.stop = dt + 1;
    L.ring.entries = de;
    L.ring.done = dd;
    L.ring.head = L.d_head;
    L.ring.exits = L.d_exits;
    L.ring.capacity = cap;
    L.ring.idle_polls = 200000;  // x ~2 us of sleep: an idle CTA leaves after ~0.5 s
    L.ring.geos = L.d_geos;
    L.ring.n_geos = 2;
    if ((e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&L.exited, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(e, "server lane stream");
    L.block = 288;
    L.smem = batch_smem(prec, 19, MAX_SLOT_NODES, L.block, 1);
    const int occ = prec == ERLBM_FP64 ? slot_server_occupancy_fp64(L.block, L.smem)
                                       : slot_server_occupancy_fp32(L.block, L.smem);
    if (occ <= 0) {
        set_error("slot loop cannot be resident%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    L.grid = std::max(1, std::min(s->desc.slot_ctas, occ * s->sms));
    return ERLBM_OK;
}

int lane_launch(SlotLane &L)
{
    const int rc = L.prec == ERLBM_FP64 ? launch_slot_server_fp64(L.ring, MAX_SLOT_NODES, L.grid, L.block, L.smem, 1,
                                                                  L.stream)
                                        : launch_slot_server_fp32(L.ring, MAX_SLOT_NODES, L.grid, L.block, L.smem, 1,
                                                                  L.stream);
    if (rc) return cuda_fail(cudaGetLastError(), "slot loop launch");
    cudaEventRecord(L.exited, L.stream);
    L.running = true;
    return ERLBM_OK;
}

// A resident loop that cannot be launched cannot serve what was published to it: those requests end
// with the launch's error.
template <class Lane>
void fail_outstanding(erlbm_server *s, Lane &L, int rc, int lane)
{
    for (const int idx : L.outstanding) {
        auto it = L.ticket_of.find(idx);
        if (it == L.ticket_of.end()) continue;
        finish(s, it->second, error_result(rc, lane));
        L.ticket_of.erase(it);
    }
    L.outstanding.clear();
}

int lane_submit(erlbm_server *s, SlotLane &L, int64_t ticket, const erlbm_request &q)
{
    const int cap = s->desc.queue_capacity;
    const int idx = L.published;
    // ring full, or the entry a lap back (whose slot this one reuses) not collected yet: retry later
    if ((int)L.outstanding.size() >= cap || L.ticket_of.count(idx - cap)) return 1;
    SlotEntry &e = L.h_entries[idx % cap];
    memset(&e, 0, sizeof(e));
    e.run.R = make_relax(q.tau, q.tau_nh, q.op);
    e.run.k = shifted::make_coef(e.run.R);
    e.run.u0 = q.u0;
    e.run.n_steps = q.n_steps;
    e.run.op = q.op;
    e.geo = q.kind == ERLBM_REQ_TG_MAP_POINT ? 0 : 1;
    L.h_done[idx % cap].seq = 0;
    L.published = idx + 1;
    __atomic_store_n(&L.h_tail[0], L.published, __ATOMIC_RELEASE);
    L.ticket_of[idx] = ticket;
    L.outstanding.push_back(idx);
    return 0;
}

void lane_collect(erlbm_server *s, SlotLane &L)
{
    const int cap = s->desc.queue_capacity;
    for (size_t k = 0; k < L.outstanding.size();) {
        const int idx = L.outstanding[k];
        SlotDone &d = L.h_done[idx % cap];
        if (__atomic_load_n(&d.seq, __ATOMIC_ACQUIRE) == idx + 1) {
            erlbm_result r;
            memset(&r, 0, sizeof(r));
            r.status = (d.res.status & 8) ? ERLBM_E_UNSUPPORTED : ERLBM_OK;
            r.label = d.res.label;
            r.steps_done = d.res.steps_done;
            r.decided_step = d.res.decided_step;
            r.energy = d.res.energy;
            r.margin = d.res.margin;
            r.lane = 0;
            r.t_admit = -1;
            const int64_t t = L.ticket_of[idx];
            L.ticket_of.erase(idx);
            finish(s, t, r);
            L.outstanding[k] = L.outstanding.back();
            L.outstanding.pop_back();
        } else {
            ++k;
        }
    }
    if (L.running && cudaEventQuery(L.exited) == cudaSuccess) L.running = false;
    if (!L.running && !L.outstanding.empty() && !s->stopping.load()) {
        const int rc = lane_launch(L);
        if (rc != ERLBM_OK) fail_outstanding(s, L, rc, 0);
    }
}

// ---- team lane --------------------------------------------------------------------------------

int team_setup(erlbm_server *s, TeamLane &L, int prec)
{
    L.prec = prec;
    const int occ = prec == ERLBM_FP64 ? team_server_occupancy_fp64() : team_server_occupancy_fp32();
    // one CTA (128 threads, 128 registers) per SM and precision: with both loops resident, half of each
    // SM's registers stay free for a slot loop's CTA
    const int want = s->desc.team_ctas > 0 ? s->desc.team_ctas : s->sms;
    L.grid = occ > 0 && s->desc.team_ctas >= 0 ? std::min(std::max(2, want), TEAM_MAX_GRID) : 0;
    if (L.grid < 2) {
        L.grid = 0;  // no resident team loop: these requests take the stream lane
        return ERLBM_OK;
    }
    cudaError_t e;
    if ((e = cudaHostAlloc(&L.h_entries, TEAM_CAPACITY * sizeof(TeamEntry), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc(&L.h_payload, TEAM_CAPACITY * TEAM_PAYLOAD, cudaHostAllocMapped)) != cudaSuccess ||

        (e = cudaHostAlloc(&L.h_done, TEAM_CAPACITY * sizeof(TeamDone), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc(&L.h_tail, 64, cudaHostAllocMapped)) != cudaSuccess)
        return cuda_fail(e, "team ring");
    memset(L.h_done, 0, TEAM_CAPACITY * sizeof(TeamDone));
    memset(L.h_tail, 0, 64);
    L.d_ctl = (TeamCtl *)s->arena.alloc(sizeof(TeamCtl));
    TeamQueue *q = (TeamQueue *)s->arena.alloc(sizeof(TeamQueue));
    TeamJob *jobs = (TeamJob *)s->arena.alloc(TEAM_MAX_JOBS * sizeof(TeamJob));
    if (!L.d_ctl || !q || !jobs) {
        set_error("server arena too small for the team lane%s%s", "", "");
        return ERLBM_E_OOM;
    }
    if ((e = cudaMemset(q, 0, sizeof(TeamQueue))) != cudaSuccess) return cuda_fail(e, "team queue");
    TeamEntry *de;
    unsigned char *dp;
    TeamDone *dd;
    int *dt;
    if ((e = cudaHostGetDevicePointer(&de, L.h_entries, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&dp, L.h_payload, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&dd, L.h_done, 0)) != cudaSuccess ||
        (e = cudaHostGetDevicePointer(&dt, L.h_tail, 0)) != cudaSuccess)
        return cuda_fail(e, "team ring mapping");
    TeamRing &r = L.ring;
    r.tail = dt;
    r.stop = dt + 1;
    r.entries = de;
    r.payload = dp;
    r.done = dd;
    r.payload_stride = TEAM_PAYLOAD;
    r.capacity = TEAM_CAPACITY;
    r.max_jobs = s->team_jobs;
    r.queue = q;
    r.ctl = L.d_ctl;
    r.jobs = jobs;
    r.pages = s->d_pages;
    r.arena = s->team_arena;
    r.n_pages = s->team_pages;
    r.idle_ns = 300000000LL;  // an idle launch leaves after 0.3 s
    // a run waits at most this long for the previous phase of its steps
    r.sync_ns = s->desc.team_wait_us > 0 ? 1000LL * s->desc.team_wait_us : 5000000000LL;
    if ((e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&L.exited, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(e, "team lane stream");
    return ERLBM_OK;
}

int team_launch(TeamLane &L)
{
    cudaError_t e = cudaMemsetAsync(L.d_ctl, 0, sizeof(TeamCtl), L.stream);
    if (e != cudaSuccess) return cuda_fail(e, "team lane reset");
    const int rc = L.prec == ERLBM_FP64 ? launch_team_server_fp64(L.ring, L.grid, L.stream)
                                        : launch_team_server_fp32(L.ring, L.grid, L.stream);
    if (rc) return cuda_fail(cudaGetLastError(), "team loop launch");
    cudaEventRecord(L.exited, L.stream);
    L.running = true;
    return ERLBM_OK;
}

// Layout of a team-lane run: its arena bytes (buffers, energies, tables, mask, fluid list) and its
// payload (tables, mask, fluid list) in the ring slot.  Returns false when the request does not go to
// the team lane: too large for the lane, the payload slot or the team arena.
bool team_plan(const erlbm_server *s, const erlbm_request &q, TeamEntry &e, std::vector<uint8_t> *solid_out)
{
    const TeamLane &L = s->team[q.precision == ERLBM_FP64 ? 0 : 1];
    if (L.grid < 2) return false;
    const long long max_nodes = s->desc.team_max_nodes > 0 ? s->desc.team_max_nodes : (1 << 19);
    memset(&e, 0, sizeof(e));
    std::vector<uint8_t> solid;
    switch (q.kind) {
    case ERLBM_REQ_TG2D:
        if (q.L > 512) return false;
        e.q = 9;
        e.nx = e.ny = q.L;
        e.nz = 1;
        e.init = 1;
        e.tab_len = 4 * q.L;
        e.k = 2. * M_PI / (double)q.L;
        break;
    case ERLBM_REQ_TG3D:
        if (q.L > 64) return false;
        e.q = 19;
        e.nx = e.ny = e.nz = q.L;
        e.init = 4;
        e.tab_len = 2 * q.L;
        break;
    case ERLBM_REQ_OBSTACLE: {
        int nx, ny;
        erlbm_obstacle_geometry(std::max(1, q.sx), std::max(1, q.sy), &nx, &ny, nullptr);
        if ((long long)nx * ny > (1 << 19)) return false;
        solid.resize((size_t)nx * ny);
        erlbm_obstacle_geometry(std::max(1, q.sx), std::max(1, q.sy), &nx, &ny, solid.data());
        e.q = 19;
        e.nx = nx;
        e.ny = ny;
        e.nz = 1;
        e.init = 0;
        e.check_density = 1;
        e.inlet_x = 1;
        e.outlet_x = nx - 2;
        break;
    }
    default:
        return false;
    }
    if (q.kind != ERLBM_REQ_OBSTACLE) e.inlet_x = e.outlet_x = -1;
    const long long nbox = (long long)e.nx * e.ny * e.nz, plane = (nbox + 63) / 64 * 64;
    if (nbox > max_nodes) return false;
    long long n_fluid = nbox;
    if (!solid.empty()) {
        n_fluid = 0;
        for (uint8_t v : solid) n_fluid += v ? 0 : 1;
    }
    auto al = [](long long b) { return (b + 255) / 256 * 256; };
    auto al16 = [](long long b) { return (b + 15) / 16 * 16; };
    const long long pop = (long long)e.q * plane * (q.precision == ERLBM_FP64 ? 8 : 4);
    e.off_buf1 = al(pop);
    e.off_scr = e.off_buf1 + al(pop);
    e.off_pay = e.off_scr + al((n_fluid + 4096) * 8);  // energies, then the partial sums
    e.solid_len = (int)solid.size();
    e.pay_solid = al16(e.tab_len * 8LL);
    e.pay_nof = e.pay_solid + al16(e.solid_len);
    const long long pay = al16(solid.empty() ? e.tab_len * 8LL : e.pay_nof + n_fluid * 4);
    if (pay > TEAM_PAYLOAD) return false;
    e.pay_bytes = pay;
    const long long bytes = e.off_pay + pay;
    const long long pages = (bytes + TEAM_PAGE - 1) / TEAM_PAGE;
    if (pages > s->team_pages) return false;
    e.pages = (int)pages;
    e.n_fluid = (int)n_fluid;
    e.prm.R = make_relax(q.tau, q.tau_nh, q.op);
    e.prm.k = shifted::make_coef(e.prm.R);
    e.u0 = q.u0;
    e.tau = q.tau;
    e.op = q.op;
    e.n_steps = q.n_steps;
    // nodes per work item: 2 (FP64) or 8 (FP32) per thread of a CTA; small FP64 items spread a small
    // lattice's step over more CTAs
    e.chunk = q.precision == ERLBM_FP64 ? 256 : 1024;
    if (solid_out) solid_out->swap(solid);
    return true;
}

double estimate_seconds(const erlbm_request &q);

int team_submit(erlbm_server *s, TeamLane &L, int64_t ticket, const erlbm_request &q)
{
    const int cap = TEAM_CAPACITY;
    const int idx = L.published;
    if ((int)L.outstanding.size() >= cap || L.ticket_of.count(idx - cap)) return 1;
    TeamEntry e;
    std::vector<uint8_t> solid;
    if (!team_plan(s, q, e, &solid)) return -1;
    e.est_ns = (long long)(estimate_seconds(q) * 1e9);
    // the payload slot is free: its previous request was collected
    unsigned char *pl = L.h_payload + (size_t)(idx % cap) * TEAM_PAYLOAD;
    double *tab = (double *)pl;
    const double Lx = (double)e.nx;
    if (e.init == 1) {
        const int n = e.nx;
        for (int x = 0; x < n; x++) {  // the stream lane's tables (job_admit)
            tab[x] = sin(2. * M_PI * x / Lx);
            tab[n + x] = cos(2. * M_PI * x / Lx);
            tab[2 * n + x] = cos(4. * M_PI * x / Lx);
            tab[3 * n + x] = cos(e.k * x);
        }
    } else if (e.init == 4) {
        const int n = e.nx;
        for (int x = 0; x < n; x++) {
            tab[x] = sin(2. * M_PI * (double)x / Lx);
            tab[n + x] = cos(2. * M_PI * (double)x / Lx);
        }
    }
    if (!solid.empty()) {
        memcpy(pl + e.pay_solid, solid.data(), solid.size());
        int *nof = (int *)(pl + e.pay_nof);
        int k = 0;
        for (size_t i = 0; i < solid.size(); i++)
            if (!solid[i]) nof[k++] = (int)i;
    }
    L.h_entries[idx % cap] = e;
    L.h_done[idx % cap].seq = 0;
    L.published = idx + 1;
    __atomic_store_n(&L.h_tail[0], L.published, __ATOMIC_RELEASE);
    L.ticket_of[idx] = ticket;
    L.outstanding.push_back(idx);
    return 0;
}

void team_collect(erlbm_server *s, TeamLane &L)
{
    const int cap = TEAM_CAPACITY;
    for (size_t k = 0; k < L.outstanding.size();) {
        const int idx = L.outstanding[k];
        TeamDone &d = L.h_done[idx % cap];
        if (__atomic_load_n(&d.seq, __ATOMIC_ACQUIRE) == idx + 1) {
            erlbm_result r;
            memset(&r, 0, sizeof(r));
            r.status = d.status ? ERLBM_E_TIMEOUT : ERLBM_OK;  // TEAM_TIMEOUT: a phase wait ran out
            r.label = d.label;
            r.steps_done = d.steps_done;
            r.decided_step = d.decided_step;
            r.energy = d.energy;
            r.margin = d.margin;
            r.lane = 2;
            r.t_admit = (double)d.t_admit_ns * 1e-9 + s->team_clock;
            const int64_t t = L.ticket_of[idx];
            L.ticket_of.erase(idx);
            finish(s, t, r);
            L.outstanding[k] = L.outstanding.back();
            L.outstanding.pop_back();
        } else {
            ++k;
        }
    }
    if (L.running && cudaEventQuery(L.exited) == cudaSuccess) L.running = false;
    if (!L.running && !L.outstanding.empty() && !s->stopping.load()) {
        const int rc = team_launch(L);
        if (rc != ERLBM_OK) fail_outstanding(s, L, rc, 2);
    }
}

// ---- stream lane ------------------------------------------------------------------------------

void job_free(erlbm_server *s, Job *j)
{
    for (void *p : j->mem) s->arena.release(p);
    j->mem.clear();
}

void *job_alloc(erlbm_server *s, Job *j, size_t bytes)
{
    void *p = s->arena.alloc(bytes);
    if (p) j->mem.push_back(p);
    return p;
}

// Builds a job; returns 0 (admitted), 1 (does not fit now), or an error code.
int job_admit(erlbm_server *s, int64_t ticket, const erlbm_request &q, Job **out)
{
    std::unique_ptr<Job> j(new Job());
    j->ticket = ticket;
    j->req = q;
    j->prec = q.precision;
    std::vector<uint8_t> solid;
    double u_in = 0.0;
    switch (q.kind) {
    case ERLBM_REQ_TG2D:
        j->q = 9;
        j->g.nx = j->g.ny = q.L;
        j->g.nz = 1;
        break;
    case ERLBM_REQ_TG3D:
    case ERLBM_REQ_TG_MAP_POINT:
        j->q = 19;
        j->g.nx = j->g.ny = q.L;
        j->g.nz = q.kind == ERLBM_REQ_TG3D ? q.L : 1;
        break;
    case ERLBM_REQ_OBSTACLE: {
        int nx, ny;
        erlbm_obstacle_geometry(std::max(1, q.sx), std::max(1, q.sy), &nx, &ny, nullptr);
        solid.resize((size_t)nx * ny);
        erlbm_obstacle_geometry(std::max(1, q.sx), std::max(1, q.sy), &nx, &ny, solid.data());
        j->q = 19;
        j->g.nx = nx;
        j->g.ny = ny;
        j->g.nz = 1;
        u_in = q.u0;
        j->check_density = true;
        break;
    }
    default:
        return ERLBM_E_INVAL;
    }
    j->g.nbox = (long long)j->g.nx * j->g.ny * j->g.nz;
    j->g.plane = (j->g.nbox + 63) / 64 * 64;
    const size_t elem = j->prec == ERLBM_FP64 ? 8 : 4;
    const size_t pop = (size_t)j->q * j->g.plane * elem;
    std::vector<int> nof;
    j->n_fluid = j->g.nbox;
    if (!solid.empty()) {
        for (long long k = 0; k < j->g.nbox; k++)
            if (!solid[k]) nof.push_back((int)k);
        j->n_fluid = (long long)nof.size();
    }
    // the initial state's table of sines and cosines along x (Taylor-Green kinds)
    std::vector<double> tab;
    int kind = 0;
    double k = 0;
    const double L = (double)j->g.nx;
    if (q.kind == ERLBM_REQ_TG2D) {
        kind = 1;
        const int n = j->g.nx;
        k = 2. * M_PI / L;
        tab.resize(4 * n);
        for (int x = 0; x < n; x++) {
            tab[x] = sin(2. * M_PI * x / L);
            tab[n + x] = cos(2. * M_PI * x / L);
            tab[2 * n + x] = cos(4. * M_PI * x / L);
            tab[3 * n + x] = cos(k * x);
        }
    } else if (q.kind == ERLBM_REQ_TG3D || q.kind == ERLBM_REQ_TG_MAP_POINT) {
        kind = 4;
        const int n = j->g.nx;
        tab.resize(2 * n);
        for (int x = 0; x < n; x++) {
            tab[x] = sin(2. * M_PI * (double)x / L);
            tab[n + x] = cos(2. * M_PI * (double)x / L);
        }
    }
    const size_t tab_bytes = std::max<size_t>(tab.size(), 1) * 8;
    const size_t need = 2 * pop + ((size_t)j->n_fluid + 4096) * 8 + 256 + solid.size() + nof.size() * 4 + tab_bytes;
    if (need > s->arena.size()) return ERLBM_E_OOM;
    if (s->arena.size() - s->arena.used() < need) return 1;
    j->buf[0] = job_alloc(s, j.get(), pop);
    j->buf[1] = job_alloc(s, j.get(), pop);
    j->scr = (double *)job_alloc(s, j.get(), ((size_t)j->n_fluid + 4096) * 8);
    j->status = (RunStatus *)job_alloc(s, j.get(), 256);
    j->tab = (double *)job_alloc(s, j.get(), tab_bytes);
    if (!solid.empty()) {
        j->solid = (uint8_t *)job_alloc(s, j.get(), solid.size());
        j->nof = (int *)job_alloc(s, j.get(), nof.size() * 4);
    }
    for (void *p : j->mem)
        if (!p) {
            job_free(s, j.get());
            return 1;  // fragmented: retry later
        }
    if (s->streams.empty()) {
        job_free(s, j.get());
        return 1;
    }
    j->slot = s->streams.back();
    s->streams.pop_back();
    j->stream = j->slot->stream;
    j->ev = j->slot->ev;
    j->h_out = j->slot->h_out;
    j->g.solid = j->solid;
    j->bc.inlet_x = j->bc.outlet_x = -1;
    j->bc.u_in = 0;
    j->bc.rho_out = 1.0;
    j->bc.inlet_kind = j->bc.outlet_kind = 0;
    j->bc.open_y = -1;
    j->bc.profile = nullptr;
    if (q.kind == ERLBM_REQ_OBSTACLE) {
        j->bc.inlet_x = 1;
        j->bc.outlet_x = j->g.nx - 2;
        j->bc.u_in = u_in;
    }
    j->R = make_relax(q.tau, q.tau_nh, q.op);
    cudaStream_t st = j->stream;
    if (!solid.empty()) {
        cudaMemcpyAsync(j->solid, solid.data(), solid.size(), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(j->nof, nof.data(), nof.size() * 4, cudaMemcpyHostToDevice, st);
    }
    RunStatus st0{0, 0x7fffffff, 0ull};
    cudaMemcpyAsync(j->status, &st0, sizeof(st0), cudaMemcpyHostToDevice, st);
    // initial populations on the device
    if (!tab.empty()) cudaMemcpyAsync(j->tab, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, st);
    const int irc = j->prec == ERLBM_FP64
                        ? launch_init_fp64(kind, j->q, j->g, (double *)j->buf[0], j->tab, q.u0, q.tau, k, 1.0, st)
                        : launch_init_fp32(kind, j->q, j->g, (float *)j->buf[0], j->tab, q.u0, q.tau, k, 1.0, st);
    // the copies above read local host vectors: they finish before this returns
    cudaStreamSynchronize(st);
    if (irc) {
        s->streams.push_back(j->slot);
        job_free(s, j.get());
        return ERLBM_E_INVAL;
    }
    j->cur = 0;
    j->kind = 0;
    j->t_admit = s->now();
    *out = j.release();
    return 0;
}

int job_enqueue_chunk(Job *j, int chunk)
{
    const long long left = j->req.n_steps - j->steps_done;
    const int m = (int)std::min<long long>(left, chunk);
    for (int s = 0; s < m; s++) {
        StepArgs a;
        a.mode = j->kind == 0 ? 1 : 0;
        a.step_index = (int)j->steps_done;
        a.check_density = j->check_density ? 1 : 0;
        a.density_limit = 10.0;
        a.status = j->check_density ? j->status : nullptr;
        a.stop_on_flag = j->check_density ? 1 : 0;
        void *src = j->buf[j->cur], *dst = j->buf[j->cur ^ 1];
        int rc;
        const bool plain = j->bc.inlet_x < 0 && j->bc.outlet_x < 0 && !j->check_density && a.mode == 0;
        if (j->prec == ERLBM_FP32_SHIFTED && j->q == 9 && plain && periodic_d2q9_fp32_ok(j->g))
            rc = launch_periodic_d2q9_fp32(j->req.op, j->g, j->R, (const float *)src, (float *)dst, j->stream);
        else if (j->prec == ERLBM_FP64)
            rc = launch_step_fp64(j->q, j->req.op, j->g, j->bc, j->R, a, (const double *)src, (double *)dst,
                                  j->stream);
        else
            rc = launch_step_fp32(j->q, j->req.op, j->g, j->bc, j->R, a, (const float *)src, (float *)dst,
                                  j->stream);
        if (rc) return ERLBM_E_CUDA;
        j->cur ^= 1;
        j->kind = 1;
        j->steps_done++;
    }
    if (j->check_density)
        cudaMemcpyAsync(j->h_out + 2, j->status, sizeof(RunStatus), cudaMemcpyDeviceToHost, j->stream);
    cudaEventRecord(j->ev, j->stream);
    j->in_flight = true;
    return ERLBM_OK;
}

// Final kinetic energy of the post-stream populations (the state the next step would start from).
int job_enqueue_final(Job *j)
{
    const void *buf = j->buf[j->cur];
    if (j->kind == 1) {
        void *spare = j->buf[j->cur ^ 1];
        const int rc = j->prec == ERLBM_FP64
                           ? launch_stream_only_fp64(j->q, j->g, (const double *)buf, (double *)spare, j->stream)
                           : launch_stream_only_fp32(j->q, j->g, (const float *)buf, (float *)spare, j->stream);
        if (rc) return ERLBM_E_CUDA;
        buf = spare;
    }
    int rc = j->prec == ERLBM_FP64 ? launch_node_fields_fp64(j->q, j->g, j->n_fluid, j->nof, (const double *)buf,
                                                             j->scr, nullptr, nullptr, j->stream)
                                   : launch_node_fields_fp32(j->q, j->g, j->n_fluid, j->nof, (const float *)buf,
                                                             j->scr, nullptr, nullptr, j->stream);
    if (rc) return ERLBM_E_CUDA;
    rc = launch_sum(j->scr, j->n_fluid, 1 << 16, j->scr + j->n_fluid, j->scr + j->n_fluid + 2048, j->stream);
    if (rc) return ERLBM_E_CUDA;
    cudaMemcpyAsync(j->h_out, j->scr + j->n_fluid + 2048, 8, cudaMemcpyDeviceToHost, j->stream);
    cudaEventRecord(j->ev, j->stream);
    j->in_flight = true;
    j->finalizing = true;
    return ERLBM_OK;
}

void job_release(erlbm_server *s, Job *j)
{
    cudaStreamSynchronize(j->stream);
    s->streams.push_back(j->slot);
    job_free(s, j);
    delete j;
}

// Advances one job; returns true when it is finished (and released).
bool job_progress(erlbm_server *s, Job *j, int chunk)
{
    if (j->in_flight) {
        const cudaError_t q = cudaEventQuery(j->ev);
        if (q == cudaErrorNotReady) return false;
        j->in_flight = false;
        if (q != cudaSuccess) {
            erlbm_result r = error_result(cuda_fail(q, "stream lane"), 1);
            finish(s, j->ticket, r);
            job_release(s, j);
            return true;
        }
    }
    if (j->finalizing) {
        erlbm_result r;
        memset(&r, 0, sizeof(r));
        r.status = ERLBM_OK;
        r.energy = j->h_out[0];
        r.steps_done = (int)j->steps_done;
        r.decided_step = j->req.n_steps;
        r.lane = 1;
        r.t_admit = j->t_admit;
        if (j->check_density) {
            RunStatus st;
            memcpy(&st, j->h_out + 2, sizeof(st));
            double mx;
            memcpy(&mx, &st.max_abs_rho_bits, sizeof(mx));
            r.margin = (st.flags & 2) ? INFINITY : mx / 10.0;
            if (st.flags) {
                r.label = 1;
                r.decided_step = st.decided_step;
                r.steps_done = st.decided_step + 1;
            }
        }
        finish(s, j->ticket, r);
        job_release(s, j);
        return true;
    }
    bool stop = j->steps_done >= j->req.n_steps;
    if (j->check_density && j->steps_done > 0) {
        RunStatus st;
        memcpy(&st, j->h_out + 2, sizeof(st));
        if (st.flags) {
            // launches after the failing step did nothing: roll the buffer index back to that step
            const long long extra = j->steps_done - (st.decided_step + 1);
            if (extra & 1) j->cur ^= 1;
            j->steps_done = st.decided_step + 1;
            stop = true;
        }
    }
    if (stop || s->stopping.load()) {
        if (job_enqueue_final(j) != ERLBM_OK) {
            finish(s, j->ticket, error_result(ERLBM_E_CUDA, 1));
            job_release(s, j);
            return true;
        }
        return false;
    }
    if (job_enqueue_chunk(j, chunk) != ERLBM_OK) {
        finish(s, j->ticket, error_result(ERLBM_E_CUDA, 1));
        job_release(s, j);
        return true;
    }
    return false;
}

// Estimated GPU seconds of a stream-lane run: lattice updates at a nominal rate (FP64 ~30x the cost
// of FP32 on GB300's FP64 pipe, D3Q19 ~2x D2Q9), with a floor per step for small lattices, whose
// chunks of steps are bound by launch latency.  It only orders admission.
double estimate_seconds(const erlbm_request &q)
{
    double nodes = 0;
    int qv = 19;
    switch (q.kind) {
    case ERLBM_REQ_TG2D:
        nodes = (double)q.L * q.L;
        qv = 9;
        break;
    case ERLBM_REQ_TG3D:
        nodes = (double)q.L * q.L * q.L;
        break;
    case ERLBM_REQ_OBSTACLE: {
        int nx = 0, ny = 0;
        erlbm_obstacle_geometry(std::max(1, q.sx), std::max(1, q.sy), &nx, &ny, nullptr);
        nodes = (double)nx * ny;
        break;
    }
    default:
        nodes = (double)q.L * q.L;
    }
    const double cost = (q.precision == ERLBM_FP64 ? 30.0 : 1.0) * (qv == 19 ? 2.0 : 1.0);
    return std::max(1, q.n_steps) * std::max(nodes * cost / 4e10, 4e-6);
}

// Admission order of the stream lane: shortest estimated work first, with aging.  The key of a
// request is its estimated GPU time minus the time it has waited, so a request that has waited
// longer than its own estimate comes before any new one: a large run is passed over for at most
// about its own run time.  The first request in that order that does not fit stops the pass, so
// memory frees up for it instead of for requests behind it.

void admit_stream_lane(erlbm_server *s)
{
    if (s->pending_b.empty()) return;
    const double now = s->now();
    std::vector<size_t> order(s->pending_b.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = k;
    auto key = [&](size_t k) {
        const Pending &p = s->pending_b[k];
        return p.est - std::max(0.0, now - p.t_submit);
    };
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key(a) < key(b); });
    std::vector<uint8_t> gone(s->pending_b.size(), 0);
    for (size_t k : order) {
        const Pending &p = s->pending_b[k];
        Job *j = nullptr;
        const int rc = job_admit(s, p.ticket, p.req, &j);
        if (rc == 1) break;
        if (rc != 0)
            finish(s, p.ticket, error_result(rc, 1));
        else
            s->active.push_back(j);
        gone[k] = 1;
    }
    size_t w = 0;
    for (size_t k = 0; k < s->pending_b.size(); k++)
        if (!gone[k]) s->pending_b[w++] = s->pending_b[k];
    s->pending_b.resize(w);
}

void scheduler(erlbm_server *s)
{
    cudaSetDevice(s->device);
    const int chunk = 64;
    for (;;) {
        std::deque<std::pair<int64_t, erlbm_request>> in;
        std::vector<double> t_in;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            const bool idle = s->active.empty() && s->pending_b.empty() && s->pending_a[0].empty() &&
                              s->pending_a[1].empty() && s->lane[0].outstanding.empty() &&
                              s->lane[1].outstanding.empty() && s->pending_c[0].empty() && s->pending_c[1].empty() &&
                              s->team[0].outstanding.empty() && s->team[1].outstanding.empty();
            if (idle && s->inbox.empty()) {
                if (s->stopping.load()) break;
                s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
            }
            in.swap(s->inbox);
            for (auto &p : in) t_in.push_back(s->t_submit[p.first]);
        }
        for (size_t k = 0; k < in.size(); k++) {
            auto &p = in[k];
            TeamEntry te;
            if (slot_eligible(p.second)) {
                s->pending_a[p.second.precision == ERLBM_FP64 ? 0 : 1].push_back(p);
            } else if (team_plan(s, p.second, te, nullptr)) {
                s->pending_c[p.second.precision == ERLBM_FP64 ? 0 : 1].push_back(p);
            } else {
                Pending q;
                q.ticket = p.first;
                q.req = p.second;
                q.t_submit = t_in[k];
                q.est = estimate_seconds(p.second);
                s->pending_b.push_back(q);
            }
        }
        // publish slot-lane requests while their ring has space
        for (int l = 0; l < 2; l++) {
            SlotLane &L = s->lane[l];
            bool any = false;
            while (!s->pending_a[l].empty() && lane_submit(s, L, s->pending_a[l].front().first,
                                                           s->pending_a[l].front().second) == 0) {
                s->pending_a[l].pop_front();
                any = true;
            }
            if (any && !L.running) {
                const int rc = lane_launch(L);
                if (rc != ERLBM_OK) fail_outstanding(s, L, rc, 0);
            }
        }
        // publish team-lane requests while their ring has space; the device admits them
        for (int l = 0; l < 2; l++) {
            TeamLane &L = s->team[l];
            bool any = false;
            while (!s->pending_c[l].empty()) {
                const int rc = team_submit(s, L, s->pending_c[l].front().first, s->pending_c[l].front().second);
                if (rc == 1) break;
                if (rc != 0) finish(s, s->pending_c[l].front().first, error_result(rc < 0 ? rc : ERLBM_E_INVAL, 2));
                s->pending_c[l].pop_front();
                any = true;
            }
            if (any && !L.running) {
                const int rc = team_launch(L);
                if (rc != ERLBM_OK) fail_outstanding(s, L, rc, 2);
            }
        }
        // admit stream-lane runs while memory and streams allow
        admit_stream_lane(s);
        for (size_t k = 0; k < s->active.size();) {
            if (job_progress(s, s->active[k], chunk)) {
                s->active[k] = s->active.back();
                s->active.pop_back();
            } else {
                ++k;
            }
        }
        lane_collect(s, s->lane[0]);
        lane_collect(s, s->lane[1]);
        team_collect(s, s->team[0]);
        team_collect(s, s->team[1]);
        if (s->stopping.load() && s->active.empty() && s->pending_b.empty() && s->pending_a[0].empty() &&
            s->pending_a[1].empty() && s->lane[0].outstanding.empty() && s->lane[1].outstanding.empty() &&
            s->pending_c[0].empty() && s->pending_c[1].empty() && s->team[0].outstanding.empty() &&
            s->team[1].outstanding.empty()) {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->inbox.empty()) break;
        }
        if (!s->active.empty() || !s->team[0].outstanding.empty() || !s->team[1].outstanding.empty())
            std::this_thread::yield();
    }
    // leave the resident loops
    for (auto &L : s->lane) {
        if (L.h_tail) __atomic_store_n(&L.h_tail[1], 1, __ATOMIC_RELEASE);
        if (L.stream) cudaStreamSynchronize(L.stream);
    }
    for (auto &L : s->team) {
        if (L.h_tail) __atomic_store_n(&L.h_tail[1], 1, __ATOMIC_RELEASE);
        if (L.stream) cudaStreamSynchronize(L.stream);
    }
}

}  // namespace

extern "C" {

int erlbm_server_start(const erlbm_server_desc *d, erlbm_server **out)
{
    if (!out) return ERLBM_E_INVAL;
    *out = nullptr;
    std::unique_ptr<erlbm_server> s(new erlbm_server());
    if (d) s->desc = *d;
    if (s->desc.hbm_budget_bytes <= 0) s->desc.hbm_budget_bytes = 8LL << 30;
    // max_streams given: it caps the team loops' runs too; by default 16 streams and 64 team runs
    if (s->desc.max_streams > 0) s->team_jobs = std::min(s->desc.max_streams, TEAM_MAX_JOBS);
    if (s->desc.max_streams <= 0) s->desc.max_streams = 16;
    if (s->desc.queue_capacity <= 0) s->desc.queue_capacity = 1 << 16;
    cudaError_t e;
    if ((e = cudaGetDevice(&s->device)) != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    if (s->desc.slot_ctas <= 0) s->desc.slot_ctas = std::max(1, s->sms / 2);
    s->t0 = Clock::now();
    int rc = s->arena.init((size_t)s->desc.hbm_budget_bytes);
    if (rc) return rc;
    // geometries of the slot lane: [0] Taylor-Green map point, [1] obstacle channel (scale 1)
    std::vector<double> tab(32);
    for (int x = 0; x < 16; x++) {
        tab[x] = sin(2. * M_PI * (double)x / 16.0);
        tab[16 + x] = cos(2. * M_PI * (double)x / 16.0);
    }
    s->d_tg_tab = (double *)s->arena.alloc(32 * 8);
    int nx, ny;
    erlbm_obstacle_geometry(1, 1, &nx, &ny, nullptr);
    std::vector<uint8_t> solid((size_t)nx * ny);
    erlbm_obstacle_geometry(1, 1, &nx, &ny, solid.data());
    s->d_obst_solid = (uint8_t *)s->arena.alloc(solid.size());
    if (!s->d_tg_tab || !s->d_obst_solid) return ERLBM_E_OOM;
    if ((e = cudaMemcpy(s->d_tg_tab, tab.data(), 32 * 8, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_obst_solid, solid.data(), solid.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "server tables");
    BatchGeo &tg = s->geos_host[0];
    memset(&tg, 0, sizeof(tg));
    tg.nx = tg.ny = 16;
    tg.nb = 256;
    tg.inlet_x = tg.outlet_x = -1;
    tg.rho0 = 1.0;
    tg.energy_every = 100;
    tg.energy_factor = 2.0;
    tg.init = INIT_TG_MAP;
    density_bounds(tg);
    tg.sinx = s->d_tg_tab;
    tg.cosx = s->d_tg_tab + 16;
    BatchGeo &ob = s->geos_host[1];
    memset(&ob, 0, sizeof(ob));
    ob.nx = nx;
    ob.ny = ny;
    ob.nb = nx * ny;
    ob.solid = s->d_obst_solid;
    ob.inlet_x = 1;
    ob.outlet_x = nx - 2;
    ob.rho0 = 1.0;
    ob.density_check = 1;
    ob.density_limit = 10.0;
    ob.init = INIT_REST;
    density_bounds(ob);
    if ((rc = lane_setup(s.get(), s->lane[0], ERLBM_FP64))) return rc;
    if ((rc = lane_setup(s.get(), s->lane[1], ERLBM_FP32_SHIFTED))) return rc;
    // the team lanes' pages: half of the budget
    s->team_pages = (int)std::min<long long>(s->desc.hbm_budget_bytes / 2 / TEAM_PAGE, 1 << 20);
    if (s->team_pages > 0) {
        s->team_arena = (char *)s->arena.alloc((size_t)s->team_pages * TEAM_PAGE);
        const size_t words = ((size_t)s->team_pages + 31) / 32;
        s->d_pages = (unsigned *)s->arena.alloc(words * 4);
        if (!s->team_arena || !s->d_pages) return ERLBM_E_OOM;
        if ((e = cudaMemset(s->d_pages, 0, words * 4)) != cudaSuccess) return cuda_fail(e, "team pages");
        if ((rc = team_setup(s.get(), s->team[0], ERLBM_FP64))) return rc;
        if ((rc = team_setup(s.get(), s->team[1], ERLBM_FP32_SHIFTED))) return rc;
        // the device clock against the server clock, for the team lanes' admission times
        long long *h_clk = nullptr;
        if ((e = cudaMallocHost(&h_clk, 64)) != cudaSuccess) return cuda_fail(e, "team clock");
        const double t0 = s->now();
        const int crc = launch_team_clock(h_clk, s->team[0].stream ? s->team[0].stream : 0);
        e = cudaDeviceSynchronize();
        const double t1 = s->now();
        if (crc == 0 && e == cudaSuccess) s->team_clock = 0.5 * (t0 + t1) - (double)h_clk[0] * 1e-9;
        cudaFreeHost(h_clk);
    }
    for (int k = 0; k < s->desc.max_streams; k++) {
        StreamSlot *sl = new StreamSlot();
        s->all_streams.push_back(sl);
        s->streams.push_back(sl);
        if ((e = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaMallocHost(&sl->h_out, 64)) != cudaSuccess)
            return cuda_fail(e, "server streams");
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail(e, "server start");
    erlbm_server *raw = s.release();
    raw->th = std::thread(scheduler, raw);
    *out = raw;
    return ERLBM_OK;
}

double erlbm_server_clock(erlbm_server *s) { return s ? s->now() : 0.0; }

int erlbm_server_submit(erlbm_server *s, const erlbm_request *q, int64_t *ticket)
{
    if (!s || !q || !ticket) return ERLBM_E_INVAL;
    if (s->stopping.load()) return ERLBM_E_STATE;
    if (q->precision != ERLBM_FP64 && q->precision != ERLBM_FP32_SHIFTED) return ERLBM_E_INVAL;
    if (q->op != ERLBM_OP_BGK && q->op != ERLBM_OP_REG && q->op != ERLBM_OP_EXTREG &&
        !(q->op == ERLBM_OP_MRT && q->kind == ERLBM_REQ_TG2D))  // MRT is D2Q9 only
        return q->op == ERLBM_OP_MRT ? ERLBM_E_UNSUPPORTED : ERLBM_E_INVAL;
    if (q->n_steps < 0 || !(q->tau > 0) || !std::isfinite(q->tau) || !std::isfinite(q->tau_nh) || q->tau_nh == 0)
        return ERLBM_E_INVAL;
    if ((q->kind == ERLBM_REQ_TG2D || q->kind == ERLBM_REQ_TG3D) && (q->L < 2 || q->L > 4096)) return ERLBM_E_INVAL;
    if (q->kind == ERLBM_REQ_TG3D && q->L > 512) return ERLBM_E_INVAL;
    if (q->kind < ERLBM_REQ_TG2D || q->kind > ERLBM_REQ_TG3D) return ERLBM_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    const int64_t t = s->next_ticket++;
    s->t_submit[t] = s->now();
    s->inbox.emplace_back(t, *q);
    if (q->kind == ERLBM_REQ_TG_MAP_POINT) s->inbox.back().second.L = 16;
    *ticket = t;
    s->cv_work.notify_one();
    return ERLBM_OK;
}

int erlbm_server_poll(erlbm_server *s, int64_t ticket, erlbm_result *r)
{
    if (!s || !r) return ERLBM_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->results.find(ticket);
    if (it == s->results.end()) return 1;
    *r = it->second;
    return ERLBM_OK;
}

int erlbm_server_wait(erlbm_server *s, int64_t ticket, erlbm_result *r, double timeout_s)
{
    if (!s || !r) return ERLBM_E_INVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (s->results.find(ticket) == s->results.end()) {
        if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout &&
            s->results.find(ticket) == s->results.end())
            return ERLBM_E_TIMEOUT;
    }
    *r = s->results[ticket];
    return ERLBM_OK;
}

int erlbm_server_stop(erlbm_server *s)
{
    if (!s) return ERLBM_OK;
    s->stopping.store(true);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    for (auto &L : s->lane) {
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.exited) cudaEventDestroy(L.exited);
        if (L.h_entries) cudaFreeHost(L.h_entries);
        if (L.h_done) cudaFreeHost(L.h_done);
        if (L.h_tail) cudaFreeHost(L.h_tail);
    }
    for (auto &L : s->team) {
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.exited) cudaEventDestroy(L.exited);
        if (L.h_entries) cudaFreeHost(L.h_entries);
        if (L.h_payload) cudaFreeHost(L.h_payload);
        if (L.h_done) cudaFreeHost(L.h_done);
        if (L.h_tail) cudaFreeHost(L.h_tail);
    }
    for (StreamSlot *sl : s->all_streams) {
        if (sl->stream) cudaStreamDestroy(sl->stream);
        if (sl->ev) cudaEventDestroy(sl->ev);
        if (sl->h_out) cudaFreeHost(sl->h_out);
        delete sl;
    }
    delete s;
    return ERLBM_OK;
}

}  // extern "C"
