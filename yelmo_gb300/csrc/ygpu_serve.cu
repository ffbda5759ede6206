// ygpu_serve.cu -- serving loop: continuous batching of velocity solves from
// many ensemble members whose state stays on the device.
//
// One host thread per server drives the GPU. Each tick it runs one Picard
// iteration of every solve on the GPU (the pre / Krylov / post step kernels
// over the list of active instances), reads back their per-instance outputs,
// retires the finished ones and admits waiting requests into the freed slots.
// Admission runs the member's thickness step and input rebuild on the device
// and the setup step of the new instances, so they join the others at the next
// tick. Host threads submit and wait through a mutex and condition variables.
#include <cuda_runtime.h>

#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <numeric>
#include <vector>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Counter-based normal deviates for the thickness step: splitmix64 of
// (key, cell) to two uniforms, Box-Muller. Same numbers alone and in a mix.
__device__ __forceinline__ unsigned long long smix(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

unsigned long long smix_host(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_step_thickness(double* H, int n2, unsigned long long key, double sigma) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n2) return;
    const double h = H[c];
    if (!(h > 0.0)) return;
    const unsigned long long a = smix(key ^ (0x632BE59BD9B4E019ull * (unsigned long long)(2 * c + 1)));
    const unsigned long long b = smix(a);
    const double u1 = ((double)(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);   // (0,1)
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);           // [0,1)
    const double z = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    const double hn = h + sigma * z;
    H[c] = hn > 0.0 ? hn : 0.0;
}

struct Member {
    int nx = 0, ny = 0, nz = 0;
    char* slab = nullptr;
    size_t bytes = 0;
    ygpu_fields f{};
    double *H = nullptr, *z_srf = nullptr, *dzsdx = nullptr, *dzsdy = nullptr;
    double *f_ice = nullptr, *H_grnd = nullptr, *f_grnd = nullptr, *fgx = nullptr, *fgy = nullptr;
    double *taud_x = nullptr, *taud_y = nullptr, *taul_x = nullptr, *taul_y = nullptr;
    int* mask_frnt = nullptr;
    int *mask_x = nullptr, *mask_y = nullptr;
    unsigned long long steps = 0;  // requests admitted so far
    bool busy = false;
};

struct Request {
    int member = -1;
    unsigned long long seed = 0, step = 0;
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
    int state = 0;                 // 0 waiting, 1 on the GPU, 2 finished
    int status = YGPU_OK;
    ygpu_stats stats{};
};

struct Admit {
    int slot;
    Member* member;                // stable: members live in a deque
    unsigned long long key;        // thickness-step key of (seed, member, step)
};

struct Slot {
    char* scratch = nullptr;
    size_t bytes = 0;
    int req = -1;                  // request on this slot, -1 when free
    int member = -1;
    size_t work = 0;               // nx*ny*nz of the instance (queue order)
    Inst inst{};
};

}  // namespace

struct ygpu_server {
    ygpu_server_cfg cfg{};
    cudaStream_t stream = nullptr;
    int max_ctas = 1;
    int max_slots = 1;
    bool mixed = false;
    bool block = false;            // tile-block preconditioner scratch
    bool ilu = false;              // ILU(0) factor scratch (residual form, -p ilu)
    size_t max_active_nu = 0;      // admission: unknowns of the active solves
    size_t active_nu = 0;
    size_t held = 0;               // device bytes held
    std::deque<Member> members;
    std::deque<Request> requests;  // index = request id; references stay valid on growth
    std::deque<int> waiting;       // request ids in submission order
    std::vector<Slot> slots;
    std::vector<int> active;       // slots on the GPU, largest instance first
    bool active_dirty = false;
    bool plan_dirty = true;
    StepShape tick_shape;
    // device arrays
    Inst* d_insts = nullptr;       // active list
    Inst* d_new = nullptr;         // instances being admitted
    InstOut* d_out = nullptr;      // one per slot
    TeamCtl* d_ctl = nullptr;
    int* d_misc = nullptr;         // [0] finished count, [1] abort flag
    int* d_map = nullptr;          // team plan of the active list (3 * max_ctas ints)
    int* d_map_new = nullptr;      // team plan of the admitted list
    int* h_map = nullptr;
    int* h_map_new = nullptr;
    // pinned host mirrors
    Inst* h_insts = nullptr;
    Inst* h_new = nullptr;
    InstOut* h_out = nullptr;
    int* h_abort = nullptr;
    // thread
    std::thread th;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    long long ticks = 0, completed = 0;
    std::string fatal;             // set when the loop stopped on a CUDA error
};

static size_t al256(size_t b) { return ygpu_align256(b); }

static size_t member_bytes(int kind, int nx, int ny, int nz) {
    const size_t n2 = (size_t)nx * ny, n3 = n2 * nz;
    size_t b = 33 * al256(n2 * 8);                    // 2D doubles
    b += 3 * al256(n2 * 4);                            // masks
    b += (kind == YGPU_KIND_DIVA ? 8 : 2) * al256(n3 * 8);   // visc, ATT (+ 3D DIVA fields)
    b += al256((size_t)nz * 8);                        // zeta
    return b;
}

// ---------------------------------------------------------------------------
// serving loop (runs on the server thread)
// ---------------------------------------------------------------------------
static int srv_fail(ygpu_server* S, const char* what, cudaError_t e) {
    std::lock_guard<std::mutex> lk(S->mu);
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    S->fatal = buf;
    // every unfinished request ends with the error
    for (Request& r : S->requests)
        if (r.state != 2) {
            r.state = 2;
            r.status = YGPU_ERR_CUDA;
            r.t_done = now_s();
        }
    S->stop = true;
    S->cv_done.notify_all();
    return YGPU_ERR_CUDA;
}

#define SCK(call, what)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return srv_fail(S, what, e_); \
    } while (0)

// Admit waiting requests into free slots. Called with the lock held; returns
// what the device work of the admission needs (instances are filled in), so
// that it runs without the lock.
static std::vector<Admit> admit_locked(ygpu_server* S) {
    std::vector<Admit> got;
    const size_t need_max = [&] {
        size_t m = 0;
        for (const Member& M : S->members) m = std::max(m, ygpu_inst_scratch_bytes(M.nx, M.ny, M.nz, S->mixed, S->block, S->ilu));
        return m;
    }();
    for (auto it = S->waiting.begin(); it != S->waiting.end();) {
        Request& R = S->requests[*it];
        Member& M = S->members[R.member];
        if (M.busy) { ++it; continue; }
        const size_t nu = (size_t)2 * M.nx * M.ny;
        const bool idle = S->active.empty() && got.empty();
        if (!idle && S->active_nu + nu > S->max_active_nu) break;     // FIFO: wait for retirements
        const size_t need = ygpu_inst_scratch_bytes(M.nx, M.ny, M.nz, S->mixed, S->block, S->ilu);
        int s = -1;
        for (int k = 0; k < (int)S->slots.size(); k++)
            if (S->slots[k].req < 0 && S->slots[k].bytes >= need) { s = k; break; }
        if (s < 0 && (int)S->slots.size() < S->max_slots && S->held + need_max <= S->cfg.hbm_budget) {
            Slot sl;
            if (cudaMalloc((void**)&sl.scratch, need_max) == cudaSuccess) {
                sl.bytes = need_max;
                S->held += need_max;
                S->slots.push_back(sl);
                s = (int)S->slots.size() - 1;
            }
        }
        if (s < 0) {
            if (S->active.empty() && got.empty()) {
                // nothing on the GPU and no slot fits or can be made: the request cannot run
                R.state = 2;
                R.status = YGPU_ERR_ADMISSION;
                R.t_done = now_s();
                it = S->waiting.erase(it);
                S->cv_done.notify_all();
                continue;
            }
            break;                 // wait for a slot (FIFO: later requests wait too)
        }
        Slot& sl = S->slots[s];
        sl.req = *it;
        sl.member = R.member;
        sl.work = (size_t)M.nx * M.ny * M.nz;
        M.busy = true;
        S->active_nu += nu;
        R.state = 1;
        R.t_admit = now_s();
        R.step = M.steps++;
        ygpu_fill_inst(sl.inst, S->cfg.kind, &M.f);
        ygpu_inst_scratch_carve(sl.inst, sl.scratch, M.nx, M.ny, M.nz, S->mixed, S->block, S->ilu);
        sl.inst.out = S->d_out + s;
        const unsigned long long key = smix_host(R.seed) ^
                                       smix_host(0x5851F42D4C957F2Dull * ((unsigned long long)R.member + 1)) ^
                                       smix_host(0x2545F4914F6CDD1Dull * (R.step + 1));
        got.push_back(Admit{s, &M, key});
        it = S->waiting.erase(it);
    }
    return got;
}

// Launch shape of n instances (nu[q] unknowns each): one team per instance with
// CTAs in proportion to its size when they fit the GPU at once, else uniform
// teams. The plan goes through the pinned h_map into d_map on the stream.
static int plan_shape(ygpu_server* S, int n, const std::vector<size_t>& nu, int* h_map, int* d_map,
                      StepShape* sh) {
    std::vector<int> map;
    int grid = 0;
    if (n > 1 && ygpu_plan_teams(S->max_ctas, n, nu.data(), map, &grid)) {
        memcpy(h_map, map.data(), sizeof(int) * map.size());
        if (cudaMemcpyAsync(d_map, h_map, sizeof(int) * map.size(), cudaMemcpyHostToDevice, S->stream) != cudaSuccess)
            return YGPU_ERR_CUDA;
        if (ygpu_step_shape_mapped(S->cfg.device, grid, d_map, sh) == YGPU_OK) {
            ygpu_step_shape_wide(sh, std::accumulate(nu.begin(), nu.end(), (size_t)0));
            return YGPU_OK;
        }
    }
    size_t max_nu = 0;
    for (size_t v : nu) max_nu = std::max(max_nu, v);
    int n_teams, team_ctas;
    ygpu_choose_teams(S->max_ctas, n, max_nu, &n_teams, &team_ctas);
    const int r = ygpu_step_shape(S->cfg.device, n_teams, team_ctas, sh);
    if (r == YGPU_OK) ygpu_step_shape_wide(sh, std::accumulate(nu.begin(), nu.end(), (size_t)0));
    return r;
}

static int prepare_admitted(ygpu_server* S, const std::vector<Admit>& got) {
    const ygpu_server_cfg& C = S->cfg;
    const ygpu_dyn_par& P = C.par;
    for (size_t q = 0; q < got.size(); q++) {
        const Slot& sl = S->slots[got[q].slot];
        const Member& M = *got[q].member;
        const int n2 = M.nx * M.ny;
        if (C.dH_sigma > 0.0) {
            k_step_thickness<<<(n2 + 255) / 256, 256, 0, S->stream>>>(M.H, n2, got[q].key, C.dH_sigma);
            ygpu_count_launches(1);
        }
        int st = ygpu_dyn_inputs_device(S->stream, M.H, M.f.z_bed, M.f.z_sl, M.f_ice, M.H_grnd, M.z_srf, M.f_grnd,
                                        M.fgx, M.fgy, M.mask_frnt, M.dzsdx, M.dzsdy, M.taud_x, M.taud_y, M.taul_x,
                                        M.taul_y, M.f.dx, C.grad_lim, C.taud_lim, P.rho_ice, P.rho_sw, P.g,
                                        P.boundaries, M.nx, M.ny);
        if (st) return srv_fail(S, "input rebuild", cudaGetLastError());
        st = ygpu_ssa_masks_device(S->stream, M.mask_x, M.mask_y, M.mask_frnt, M.f_ice, M.f_grnd, C.lateral_bc,
                                   P.boundaries, M.nx, M.ny);
        if (st) return srv_fail(S, "mask rebuild", cudaGetLastError());
        SCK(cudaMemsetAsync(S->d_out + got[q].slot, 0, sizeof(InstOut), S->stream), "output reset");
        S->h_new[q] = sl.inst;
    }
    const int n = (int)got.size();
    SCK(cudaMemcpyAsync(S->d_new, S->h_new, sizeof(Inst) * (size_t)n, cudaMemcpyHostToDevice, S->stream), "upload");
    std::vector<size_t> nu;
    for (const Admit& a : got) nu.push_back((size_t)2 * S->slots[a.slot].inst.n2);
    StepShape sh;
    int st = plan_shape(S, n, nu, S->h_map_new, S->d_map_new, &sh);
    if (!st) st = ygpu_launch_step(YG_STEP_SETUP, S->stream, sh, S->d_new, n, P, S->d_ctl, S->d_misc, S->d_misc + 1);
    if (!st && P.ssa_iter_max == 0)
        st = ygpu_launch_step(YG_STEP_FINAL, S->stream, sh, S->d_new, n, P, S->d_ctl, S->d_misc, S->d_misc + 1);
    if (st) return srv_fail(S, "setup launch", cudaGetLastError());
    // the host staging of d_new is reused by the next admission: wait for the copy
    SCK(cudaStreamSynchronize(S->stream), "setup");
    return YGPU_OK;
}

static int run_tick(ygpu_server* S) {
    YgRange range("ygpu serve tick");
    const ygpu_dyn_par& P = S->cfg.par;
    const int n = (int)S->active.size();
    if (S->active_dirty) {
        std::stable_sort(S->active.begin(), S->active.end(),
                         [&](int a, int b) { return S->slots[a].work > S->slots[b].work; });
        for (int q = 0; q < n; q++) S->h_insts[q] = S->slots[S->active[q]].inst;
        SCK(cudaMemcpyAsync(S->d_insts, S->h_insts, sizeof(Inst) * (size_t)n, cudaMemcpyHostToDevice, S->stream),
            "active upload");
        S->active_dirty = false;
        S->plan_dirty = true;
    }
    // the plan changes with the active list only
    int st = YGPU_OK;
    if (S->plan_dirty) {
        std::vector<size_t> nu;
        for (int s : S->active) nu.push_back((size_t)2 * S->slots[s].inst.n2);
        st = plan_shape(S, n, nu, S->h_map, S->d_map, &S->tick_shape);
        S->plan_dirty = false;
    }
    const StepShape sh = S->tick_shape;
    for (int step : {YG_STEP_PRE, YG_STEP_KRYLOV, YG_STEP_POST}) {
        if (st) break;
        st = ygpu_launch_step(step, S->stream, sh, S->d_insts, n, P, S->d_ctl, S->d_misc, S->d_misc + 1);
    }
    if (st) return srv_fail(S, "step launch", cudaGetLastError());
    SCK(cudaMemcpyAsync(S->h_out, S->d_out, sizeof(InstOut) * S->slots.size(), cudaMemcpyDeviceToHost, S->stream),
        "output read");
    SCK(cudaMemcpyAsync(S->h_abort, S->d_misc + 1, sizeof(int), cudaMemcpyDeviceToHost, S->stream), "abort read");
    SCK(cudaStreamSynchronize(S->stream), "tick");
    ygpu_step_timing_flush();
    S->ticks++;
    return YGPU_OK;
}

// retire finished solves; lock held
static void retire_locked(ygpu_server* S) {
    const bool aborted = (*S->h_abort != 0);
    const double t = now_s();
    std::vector<int> keep;
    for (int s : S->active) {
        Slot& sl = S->slots[s];
        const InstOut& o = S->h_out[s];
        if (!o.done && !aborted) {
            keep.push_back(s);
            continue;
        }
        Request& R = S->requests[sl.req];
        R.state = 2;
        R.t_done = t;
        R.status = aborted ? YGPU_ERR_TIMEOUT : o.status;
        ygpu_stats& St = R.stats;
        memset(&St, 0, sizeof(St));
        St.ssa_iter_now = o.iter_now;
        St.ssa_lin_iter = o.lin_iter;
        St.ssa_lin_fail = o.lin_fail;
        St.ssa_lim_n = o.lim_n;
        St.ssa_resid = o.resid;
        St.lin_resid = o.lin_resid;
        St.outer_iter = o.outer_iter; St.active_cells = o.n_active;
        ygpu_lin_method_run_grid(&S->cfg.par, S->members[R.member].nx, S->members[R.member].ny, &St.lin_solver_run,
                                 &St.lin_precond_run);
        St.status = R.status;
        St.device_ms = (R.t_done - R.t_admit) * 1e3;
        for (int q = 0; q < 10; q++) St.phase_ms[q] = o.phase_ns[q] * 1e-6;
        S->members[R.member].busy = false;
        S->active_nu -= (size_t)2 * S->members[R.member].nx * S->members[R.member].ny;
        sl.req = -1;
        sl.member = -1;
        S->completed++;
    }
    if (keep.size() != S->active.size()) S->active_dirty = true;
    S->active.swap(keep);
    if (aborted) {
        // a device wait ran out: start the next tick from clean team state
        cudaMemsetAsync(S->d_misc, 0, 2 * sizeof(int), S->stream);
        cudaMemsetAsync(S->d_ctl, 0, sizeof(TeamCtl) * (size_t)S->max_ctas, S->stream);
        cudaStreamSynchronize(S->stream);
    }
    S->cv_done.notify_all();
}

static void serve_loop(ygpu_server* S) {
    cudaSetDevice(S->cfg.device);
    for (;;) {
        std::vector<Admit> got;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->active.empty()) {
                S->cv_work.wait_for(lk, std::chrono::milliseconds(50),
                                    [&] { return S->stop || !S->waiting.empty(); });
            }
            if (S->stop && S->active.empty()) return;
            if (!S->stop) got = admit_locked(S);
        }
        if (!got.empty()) {
            if (prepare_admitted(S, got)) return;
            std::lock_guard<std::mutex> lk(S->mu);
            for (const Admit& a : got) S->active.push_back(a.slot);
            S->active_dirty = true;
        }
        if (S->active.empty()) continue;
        if (run_tick(S)) return;
        std::lock_guard<std::mutex> lk(S->mu);
        retire_locked(S);
    }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" ygpu_server* ygpu_server_create(const ygpu_server_cfg* cfg) {
    if (!cfg) { ygpu_set_error("cfg is NULL"); return nullptr; }
    if (ygpu_check_par(&cfg->par)) return nullptr;
    if (cfg->kind != YGPU_KIND_SSA && cfg->kind != YGPU_KIND_DIVA) { ygpu_set_error("bad solver kind %d", cfg->kind); return nullptr; }
    if (cfg->dH_sigma < 0.0) { ygpu_set_error("dH_sigma must be >= 0"); return nullptr; }
    if (cudaSetDevice(cfg->device) != cudaSuccess) { ygpu_set_error("cannot use device %d", cfg->device); return nullptr; }
    // the step kernels' non-inlined phases take up to about 1.3 KB of stack per
    // thread (ptxas' cumulative stack size), above the default limit: give them 4 KB
    size_t stack = 0;
    cudaDeviceGetLimit(&stack, cudaLimitStackSize);
    if (stack < 4096) cudaDeviceSetLimit(cudaLimitStackSize, 4096);
    ygpu_server* S = new ygpu_server();
    S->cfg = *cfg;
    S->mixed = (cfg->par.precision == YGPU_PREC_MIXED);
    S->block = ygpu_wants_block(cfg->par);
    S->ilu = ygpu_wants_ilu(cfg->par);
    S->max_ctas = ygpu_solver_max_ctas(cfg->device);
    if (S->max_ctas < 1 || ygpu_init_constants(cfg->device)) {
        ygpu_set_error("solver kernels cannot be resident on device %d", cfg->device);
        delete S;
        return nullptr;
    }
    // Concurrency: every tick advances all active solves by one Picard iteration
    // and waits for the slowest linear solve among them, so fewer, larger teams
    // waste less of the tick. By default at most 1.5 M unknowns are active (256
    // uneven members of 64-321 cells a side: 116 solves/s with 16 active, 96
    // with 64, 62 with 152), and never more solves than SMs.
    S->max_slots = cfg->max_slots > 0 ? cfg->max_slots : ygpu_sm_count(cfg->device);
    S->max_active_nu = cfg->max_active_unknowns > 0 ? (size_t)cfg->max_active_unknowns : (size_t)1500000;
    if (S->max_slots > 4096) S->max_slots = 4096;
    const int ms = S->max_slots;
    bool ok = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_insts, sizeof(Inst) * ms) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_new, sizeof(Inst) * ms) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_out, sizeof(InstOut) * ms) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_ctl, sizeof(TeamCtl) * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_misc, 64) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_map, sizeof(int) * 3 * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&S->d_map_new, sizeof(int) * 3 * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_map, sizeof(int) * 3 * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_map_new, sizeof(int) * 3 * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_insts, sizeof(Inst) * ms) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_new, sizeof(Inst) * ms) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_out, sizeof(InstOut) * ms) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&S->h_abort, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMemset(S->d_ctl, 0, sizeof(TeamCtl) * (size_t)S->max_ctas) == cudaSuccess;
    ok = ok && cudaMemset(S->d_misc, 0, 64) == cudaSuccess;
    ok = ok && cudaMemset(S->d_out, 0, sizeof(InstOut) * ms) == cudaSuccess;
    if (!ok) {
        ygpu_set_error("server set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
        ygpu_server_destroy(S);
        return nullptr;
    }
    S->held = sizeof(Inst) * 2 * ms + sizeof(InstOut) * ms + sizeof(TeamCtl) * (size_t)S->max_ctas + 64 +
              2 * sizeof(int) * 3 * (size_t)S->max_ctas;
    if (S->held > cfg->hbm_budget) {
        ygpu_set_error("hbm_budget %llu is below the server's fixed %zu bytes", cfg->hbm_budget, S->held);
        ygpu_server_destroy(S);
        return nullptr;
    }
    S->th = std::thread(serve_loop, S);
    return S;
}

extern "C" void ygpu_server_destroy(ygpu_server* S) {
    if (!S) return;
    if (S->th.joinable()) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
            // requests still waiting are not started
            for (int id : S->waiting) {
                Request& R = S->requests[id];
                R.state = 2;
                R.status = YGPU_ERR_BUSY;
                R.t_done = now_s();
            }
            S->waiting.clear();
        }
        S->cv_work.notify_all();
        S->th.join();
    }
    cudaSetDevice(S->cfg.device);
    if (S->stream) cudaStreamSynchronize(S->stream);
    for (Member& M : S->members) cudaFree(M.slab);
    for (Slot& sl : S->slots) cudaFree(sl.scratch);
    cudaFree(S->d_insts);
    cudaFree(S->d_new);
    cudaFree(S->d_out);
    cudaFree(S->d_ctl);
    cudaFree(S->d_misc);
    cudaFree(S->d_map);
    cudaFree(S->d_map_new);
    cudaFreeHost(S->h_map);
    cudaFreeHost(S->h_map_new);
    cudaFreeHost(S->h_insts);
    cudaFreeHost(S->h_new);
    cudaFreeHost(S->h_out);
    cudaFreeHost(S->h_abort);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}

extern "C" int ygpu_server_add_member(ygpu_server* S, const ygpu_fields* h, int* member_id) {
    if (!S || !h || !member_id) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    if (h->nx < 3 || h->ny < 3 || h->nz < 2 || (size_t)h->nx * h->ny > (size_t)(1 << 29)) {
        ygpu_set_error("bad member grid %dx%dx%d", h->nx, h->ny, h->nz);
        return YGPU_ERR_BAD_ARG;
    }
    if (!(h->dx > 0.0) || !(h->dy > 0.0) || !(h->n_glen > 0.0)) { ygpu_set_error("dx, dy and n_glen must be positive"); return YGPU_ERR_BAD_ARG; }
    const void* need[] = {h->H_ice, h->z_bed, h->z_sl, h->c_bed, h->f_slide, h->ATT, h->zeta_aa};
    for (const void* q : need)
        if (!q) { ygpu_set_error("a member input (H_ice, z_bed, z_sl, c_bed, f_slide, ATT, zeta_aa) is NULL"); return YGPU_ERR_BAD_ARG; }
    const int kind = S->cfg.kind;
    const size_t bytes = member_bytes(kind, h->nx, h->ny, h->nz);
    const size_t scratch = ygpu_inst_scratch_bytes(h->nx, h->ny, h->nz, S->mixed, S->block, S->ilu);
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->fatal.empty()) { ygpu_set_error("server stopped: %s", S->fatal.c_str()); return YGPU_ERR_CUDA; }
    // the member and, if no slot exists yet, one slot for it must fit the budget
    const size_t slot_need = S->slots.empty() ? scratch : 0;
    if (S->held + bytes + slot_need > S->cfg.hbm_budget) {
        ygpu_set_error("member %dx%dx%d needs %zu bytes: over the HBM budget (%zu of %llu held)", h->nx, h->ny,
                       h->nz, bytes, S->held, S->cfg.hbm_budget);
        return YGPU_ERR_ADMISSION;
    }
    cudaSetDevice(S->cfg.device);
    Member M;
    M.nx = h->nx; M.ny = h->ny; M.nz = h->nz;
    if (cudaMalloc((void**)&M.slab, bytes) != cudaSuccess) {
        cudaGetLastError();
        ygpu_set_error("device allocation of %zu bytes failed", bytes);
        return YGPU_ERR_NOMEM;
    }
    M.bytes = bytes;
    const size_t n2 = (size_t)h->nx * h->ny, n3 = n2 * h->nz;
    char* p = M.slab;
    auto D = [&](size_t n) { double* r = (double*)p; p += al256(n * 8); return r; };
    auto Iv = [&](size_t n) { int* r = (int*)p; p += al256(n * 4); return r; };
    ygpu_fields& f = M.f;
    memset(&f, 0, sizeof(f));
    f.nx = h->nx; f.ny = h->ny; f.nz = h->nz; f.dx = h->dx; f.dy = h->dy; f.n_glen = h->n_glen;
    f.ux_bar = D(n2); f.uy_bar = D(n2); f.ux_b = D(n2); f.uy_b = D(n2);
    f.taub_acx = D(n2); f.taub_acy = D(n2); f.beta = D(n2); f.beta_acx = D(n2); f.beta_acy = D(n2);
    f.beta_eff = D(n2); f.visc_eff_int = D(n2); f.ssa_err_acx = D(n2); f.ssa_err_acy = D(n2);
    double* c_bed = D(n2);
    double* f_slide = D(n2);
    M.taud_x = D(n2); M.taud_y = D(n2); M.taul_x = D(n2); M.taul_y = D(n2);
    M.H = D(n2); M.f_ice = D(n2); M.H_grnd = D(n2); M.f_grnd = D(n2); M.fgx = D(n2); M.fgy = D(n2);
    double* z_sl = D(n2);
    double* z_bed = D(n2);
    M.z_srf = D(n2); M.dzsdx = D(n2); M.dzsdy = D(n2);
    M.mask_x = Iv(n2); M.mask_y = Iv(n2); M.mask_frnt = Iv(n2);
    f.visc_eff = D(n3);
    double* ATT = D(n3);
    if (kind == YGPU_KIND_DIVA) {
        f.ux = D(n3); f.uy = D(n3); f.ux_i = D(n3); f.uy_i = D(n3); f.duxdz = D(n3); f.duydz = D(n3);
    }
    double* zeta = D(h->nz);
    f.c_bed = c_bed; f.f_slide = f_slide;
    f.taud_acx = M.taud_x; f.taud_acy = M.taud_y; f.taul_int_acx = M.taul_x; f.taul_int_acy = M.taul_y;
    f.H_ice = M.H; f.f_ice = M.f_ice; f.H_grnd = M.H_grnd; f.f_grnd = M.f_grnd;
    f.f_grnd_acx = M.fgx; f.f_grnd_acy = M.fgy; f.ATT = ATT; f.zeta_aa = zeta; f.z_sl = z_sl; f.z_bed = z_bed;
    f.z_srf = M.z_srf;
    f.ssa_mask_acx = M.mask_x; f.ssa_mask_acy = M.mask_y;
    bool ok = cudaMemset(M.slab, 0, bytes) == cudaSuccess;
    auto up = [&](void* dst, const void* src, size_t b) {
        if (src && ok) ok = cudaMemcpy(dst, src, b, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    up(M.H, h->H_ice, n2 * 8);
    up(z_bed, h->z_bed, n2 * 8);
    up(z_sl, h->z_sl, n2 * 8);
    up(c_bed, h->c_bed, n2 * 8);
    up(f_slide, h->f_slide, n2 * 8);
    up(ATT, h->ATT, n3 * 8);
    up(zeta, h->zeta_aa, (size_t)h->nz * 8);
    up(f.beta, h->beta, n2 * 8);
    up(f.beta_acx, h->beta_acx, n2 * 8);
    up(f.beta_acy, h->beta_acy, n2 * 8);
    up(f.ux_b, h->ux_b, n2 * 8);
    up(f.uy_b, h->uy_b, n2 * 8);
    up(f.taub_acx, h->taub_acx, n2 * 8);
    up(f.taub_acy, h->taub_acy, n2 * 8);
    if (kind == YGPU_KIND_DIVA) {
        up(f.ux_bar, h->ux_bar, n2 * 8);
        up(f.uy_bar, h->uy_bar, n2 * 8);
    }
    if (h->visc_eff) {
        up(f.visc_eff, h->visc_eff, n3 * 8);
    } else if (ok) {
        std::vector<double> v(n3, 1e5);
        ok = cudaMemcpy(f.visc_eff, v.data(), n3 * 8, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        ygpu_set_error("member upload failed: %s", cudaGetErrorString(cudaGetLastError()));
        cudaFree(M.slab);
        return YGPU_ERR_CUDA;
    }
    S->held += bytes;
    *member_id = (int)S->members.size();
    S->members.push_back(M);
    return YGPU_OK;
}

extern "C" int ygpu_server_submit(ygpu_server* S, int member, unsigned long long seed, int* request_id) {
    if (!S || !request_id) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (!S->fatal.empty()) { ygpu_set_error("server stopped: %s", S->fatal.c_str()); return YGPU_ERR_CUDA; }
        if (S->stop) { ygpu_set_error("server is stopping"); return YGPU_ERR_BUSY; }
        if (member < 0 || member >= (int)S->members.size()) { ygpu_set_error("bad member %d", member); return YGPU_ERR_BAD_ARG; }
        Request R;
        R.member = member;
        R.seed = seed;
        R.t_submit = now_s();
        *request_id = (int)S->requests.size();
        S->requests.push_back(R);
        S->waiting.push_back(*request_id);
    }
    S->cv_work.notify_one();
    return YGPU_OK;
}

extern "C" int ygpu_server_poll(ygpu_server* S, int id) {
    if (!S) return YGPU_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (id < 0 || id >= (int)S->requests.size()) return YGPU_ERR_BAD_ARG;
    return S->requests[id].state == 2 ? 1 : 0;
}

extern "C" int ygpu_server_wait(ygpu_server* S, int id, double timeout_s, ygpu_stats* stats, double* latency_ms) {
    if (!S) { ygpu_set_error("server is NULL"); return YGPU_ERR_BAD_ARG; }
    std::unique_lock<std::mutex> lk(S->mu);
    if (id < 0 || id >= (int)S->requests.size()) { ygpu_set_error("bad request id %d", id); return YGPU_ERR_BAD_ARG; }
    auto done = [&] { return S->requests[id].state == 2; };
    if (timeout_s < 0.0) S->cv_done.wait(lk, done);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) return YGPU_ERR_BUSY;
    const Request& R = S->requests[id];
    if (stats) *stats = R.stats;
    if (latency_ms) *latency_ms = (R.t_done - R.t_submit) * 1e3;
    if (R.status == YGPU_ERR_CUDA && !S->fatal.empty()) ygpu_set_error("server stopped: %s", S->fatal.c_str());
    if (R.status == YGPU_ERR_ADMISSION) ygpu_set_error("no solve slot fits the HBM budget");
    return R.status;
}

extern "C" int ygpu_server_fetch(ygpu_server* S, int member, int field, double* host) {
    if (!S || !host) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    if (member < 0 || member >= (int)S->members.size()) { ygpu_set_error("bad member %d", member); return YGPU_ERR_BAD_ARG; }
    const Member& M = S->members[member];
    if (M.busy) { ygpu_set_error("member %d is solving", member); return YGPU_ERR_BUSY; }
    const size_t n2 = (size_t)M.nx * M.ny;
    const bool diva = (S->cfg.kind == YGPU_KIND_DIVA);
    const double* src = nullptr;
    size_t n = n2;
    switch (field) {
        case YGPU_SRV_UX: src = diva ? M.f.ux_bar : M.f.ux_b; break;
        case YGPU_SRV_UY: src = diva ? M.f.uy_bar : M.f.uy_b; break;
        case YGPU_SRV_VISC: src = M.f.visc_eff; n = n2 * M.nz; break;
        case YGPU_SRV_H: src = M.H; break;
        case YGPU_SRV_UXB: src = M.f.ux_b; break;
        case YGPU_SRV_UYB: src = M.f.uy_b; break;
        case YGPU_SRV_TAUBX: src = M.f.taub_acx; break;
        case YGPU_SRV_TAUBY: src = M.f.taub_acy; break;
        case YGPU_SRV_BETA: src = M.f.beta; break;
        case YGPU_SRV_BETAX: src = M.f.beta_acx; break;
        case YGPU_SRV_BETAY: src = M.f.beta_acy; break;
        default: ygpu_set_error("bad field code %d", field); return YGPU_ERR_BAD_ARG;
    }
    cudaSetDevice(S->cfg.device);
    if (cudaMemcpy(host, src, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        ygpu_set_error("fetch failed: %s", cudaGetErrorString(cudaGetLastError()));
        return YGPU_ERR_CUDA;
    }
    return YGPU_OK;
}

extern "C" int ygpu_server_member_steps(ygpu_server* S, int member, unsigned long long* steps) {
    if (!S || !steps) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    if (member < 0 || member >= (int)S->members.size()) { ygpu_set_error("bad member %d", member); return YGPU_ERR_BAD_ARG; }
    *steps = S->members[member].steps;
    return YGPU_OK;
}

extern "C" int ygpu_server_set_member_steps(ygpu_server* S, int member, unsigned long long steps) {
    if (!S) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    if (member < 0 || member >= (int)S->members.size()) { ygpu_set_error("bad member %d", member); return YGPU_ERR_BAD_ARG; }
    Member& M = S->members[member];
    bool waiting = M.busy;
    for (int id : S->waiting) waiting = waiting || (S->requests[id].member == member);
    if (waiting) { ygpu_set_error("member %d has a request waiting or solving", member); return YGPU_ERR_BUSY; }
    M.steps = steps;
    return YGPU_OK;
}

extern "C" int ygpu_server_get_info(ygpu_server* S, ygpu_server_info* info) {
    if (!S || !info) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    info->members = (int)S->members.size();
    info->slots = (int)S->slots.size();
    info->active = (int)S->active.size();
    info->pending = (int)S->waiting.size();
    info->ticks = S->ticks;
    info->completed = S->completed;
    info->bytes_held = S->held;
    return YGPU_OK;
}
