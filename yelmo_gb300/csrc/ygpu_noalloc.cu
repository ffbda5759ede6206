// ygpu_noalloc.cu -- a solve entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a Fortran or C host whose device memory
// is owned by another runtime or by a pool allocator that must see every
// allocation, or a long-running server that must not grow its footprint after
// start-up. ygpu_solve_device_noalloc solves one instance on device-resident
// fields the caller passes, with the same kernels and the same answer as
// ygpu_solve_device, but keeps all of its scratch (instance descriptor, team
// control block, Krylov vectors, viscosity buffers) in the file-scope array
// below instead of a context arena. It has no neff hook: with a hook set on the
// calling thread, a DIVA solve is refused (the hook's per-iteration round trip
// belongs to the context entry points).
//
// The first call on a device also checks that the step kernels' stack (ptxas'
// cumulative stack size, about 1 KB per thread) fits the context's stack
// limit; it does not raise the limit, since that reserves device memory.
//
// The array has a fixed size, YGPU_NOALLOC_SCRATCH_BYTES (64 MiB), and every
// GPU that loads this library holds it until the process exits. Its device
// address is obtained once per device with cudaGetSymbolAddress, with that
// device current, on the first call on that device; host code never passes
// the symbol itself to a kernel (in host code it names a host-side stand-in,
// not device memory).
//
// All calls share the one array and it keeps the contents of the last call:
// the control words that must start at zero are cleared on every call, and two
// calls that overlap on the GPU (different host threads or streams at the same
// time) race on it. The call is stream-ordered on the caller's stream and
// returns after that stream has finished the solve.
#include <cuda_runtime.h>

#include <string.h>

#include <mutex>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[YGPU_NOALLOC_SCRATCH_BYTES];

namespace {
struct DeviceSetup {
    bool done = false;
    char* base = nullptr;          // device address of g_noalloc_scratch
    int max_ctas = 0;
};
DeviceSetup g_setup[64];
std::mutex g_setup_mu;
}  // namespace

static int noalloc_setup(int dev, DeviceSetup** out) {
    if (dev < 0 || dev >= 64) {
        ygpu_set_error("device index %d out of range", dev);
        return YGPU_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceSetup& S = g_setup[dev];
    if (!S.done) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            ygpu_set_error("cudaGetSymbolAddress of the scratch array failed on device %d: %s", dev,
                           cudaGetErrorString(e));
            return YGPU_ERR_CUDA;
        }
        S.base = (char*)p;
        S.max_ctas = ygpu_solver_max_ctas(dev);
        // the step kernels' stack must fit the context's stack limit: raising it
        // would reserve device memory, which this entry point does not do
        size_t limit = 0;
        cudaDeviceGetLimit(&limit, cudaLimitStackSize);
        const size_t need = ygpu_solver_stack_bytes();
        if (need > limit) {
            ygpu_set_error("the solver kernels need %zu bytes of stack per thread, the context allows %zu: create "
                           "a context (ygpu_ctx_create) once, or raise cudaLimitStackSize, before this call",
                           need, limit);
            return YGPU_ERR_CUDA;
        }
        if (S.max_ctas < 1) {
            ygpu_set_error("solver kernel cannot be resident on device %d", dev);
            return YGPU_ERR_CUDA;
        }
        S.done = true;
    }
    *out = &S;
    return YGPU_OK;
}

extern "C" int ygpu_solve_device_noalloc(int kind, const ygpu_dyn_par* par, const ygpu_fields* f,
                                         ygpu_stats* stats, void* stream) {
    int st = ygpu_check_par(par);
    if (st) return st;
    if (kind != YGPU_KIND_SSA && kind != YGPU_KIND_DIVA) {
        ygpu_set_error("bad solver kind %d", kind);
        return YGPU_ERR_BAD_ARG;
    }
    if ((st = ygpu_fields_check(kind, f))) return st;
    if (kind == YGPU_KIND_DIVA && ygpu_neff_hook_is_set()) {
        ygpu_set_error("a neff hook is set on this thread: the allocation-free entry point does not run it "
                       "(use ygpu_solve_device or ygpu_calc_velocity_diva, or clear the hook)");
        return YGPU_ERR_BAD_ARG;
    }
    // the call reads the count of finished solves back and synchronises its
    // stream, which a stream capture forbids: refuse before enqueueing anything
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        const cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
        if (ce != cudaSuccess) cudaGetLastError();
        if (ce != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            ygpu_set_error("the stream is being captured: the allocation-free entry point synchronises its "
                           "stream and cannot be recorded into a CUDA graph");
            return YGPU_ERR_BAD_ARG;
        }
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        ygpu_set_error("cudaGetDevice failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    DeviceSetup* S = nullptr;
    if ((st = noalloc_setup(dev, &S))) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const bool mixed = (par->precision == YGPU_PREC_MIXED);

    // layout inside the array: descriptor, outputs, team control, queue/abort, instance scratch
    const size_t off_inst = 0;
    const size_t off_out = ygpu_align256(off_inst + ygpu_inst_bytes());
    const size_t off_ctl = ygpu_align256(off_out + sizeof(InstOut));
    const size_t off_misc = ygpu_align256(off_ctl + ygpu_teamctl_bytes());
    const size_t off_arena = ygpu_align256(off_misc + 2 * sizeof(int));
    const size_t need = off_arena + ygpu_inst_scratch_bytes(f->nx, f->ny, f->nz, mixed, ygpu_wants_block(*par),
                                                            ygpu_wants_ilu(*par));
    if (need > (size_t)YGPU_NOALLOC_SCRATCH_BYTES) {
        ygpu_set_error("instance %dx%dx%d needs %zu bytes of scratch, more than the %zu of the "
                       "allocation-free entry point (use ygpu_solve_device)",
                       f->nx, f->ny, f->nz, need, (size_t)YGPU_NOALLOC_SCRATCH_BYTES);
        return YGPU_ERR_BAD_ARG;
    }
    char* base = S->base;
    Inst h;
    ygpu_fill_inst(h, kind, f);
    ygpu_inst_scratch_carve(h, base + off_arena, f->nx, f->ny, f->nz, mixed, ygpu_wants_block(*par),
                            ygpu_wants_ilu(*par));
    InstOut* d_out = (InstOut*)(base + off_out);
    h.out = d_out;
    Inst* d_inst = (Inst*)(base + off_inst);
    TeamCtl* d_ctl = (TeamCtl*)(base + off_ctl);
    int* d_misc = (int*)(base + off_misc);
    if ((e = cudaMemcpyAsync(d_inst, &h, sizeof(Inst), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_out, 0, sizeof(InstOut), s)) != cudaSuccess) {
        ygpu_set_error("scratch set-up failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    const int team_ctas = ygpu_single_team_ctas(S->max_ctas, (size_t)2 * f->nx * f->ny);
    // ygpu_launch_solver clears the team control block, the queue and the abort flag
    st = ygpu_launch_solver(dev, s, d_inst, 1, *par, d_ctl, 1, team_ctas, d_misc, d_misc + 1);
    if (st) return st;
    InstOut o;
    int abort_flag = 0;
    if ((e = cudaMemcpyAsync(&o, d_out, sizeof(InstOut), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&abort_flag, d_misc + 1, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        ygpu_set_error("solve failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    const int status = abort_flag ? YGPU_ERR_TIMEOUT : o.status;
    if (abort_flag) ygpu_set_error("a device-side wait hit its iteration limit (team barrier timeout)");
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->ssa_iter_now = o.iter_now;
        stats->ssa_lin_iter = o.lin_iter;
        stats->ssa_lin_fail = o.lin_fail;
        stats->ssa_lim_n = o.lim_n;
        stats->ssa_resid = o.resid;
        stats->lin_resid = o.lin_resid;
        stats->outer_iter = o.outer_iter; stats->active_cells = o.n_active;
        ygpu_lin_method_run_grid(par, f->nx, f->ny, &stats->lin_solver_run, &stats->lin_precond_run);
        stats->status = status;
        for (int q = 0; q < 10; q++) stats->phase_ms[q] = o.phase_ns[q] * 1e-6;
    }
    return status;
}
