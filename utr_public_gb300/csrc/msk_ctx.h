// msk_ctx.h -- the library context and the host helpers shared by the
// translation units of libmsk (the multislice host code and the UTR
// reconstruction): device buffers, per-kernel accounting, error reporting,
// the TMA views of the column passes and the device error flags.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "msk.h"
#include "msk_launch.cuh"
#include "msk_types.h"

namespace msk {

// Device allocations made by the library in this process (every one goes
// through DevBuf::reserve); msk_device_allocations() reports it.
extern std::atomic<long long> g_device_allocs;
// Set on a host thread while a call that must not allocate runs on it
// (msk_calculate_static): a DevBuf that would have to grow fails instead.
extern thread_local bool t_no_alloc;

// A device allocation that only grows -- or, when `borrowed`, a view of
// memory the library does not own (a region of a fixed array), which never
// grows and is never freed.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool borrowed = false;
    cudaError_t reserve(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        if (borrowed || t_no_alloc) return cudaErrorMemoryAllocation;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) {
            cap = bytes;
            g_device_allocs.fetch_add(1, std::memory_order_relaxed);
        }
        return e;
    }
    // a view of `bytes` bytes at `q`, owned elsewhere
    void borrow(void *q, size_t bytes)
    {
        p = q;
        cap = bytes;
        borrowed = true;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
    void release()
    {
        if (p && !borrowed) cudaFree(p);
        p = nullptr;
        cap = 0;
        borrowed = false;
    }
};

// Kinds of launches for the per-kernel accounting (msk_profile).
enum Kind {
    kSplat, kKColMask, kTransmit, kKColProp, kFresnel, kIntensity, kExit, kInit, kPlane, kFresTab,
    kExpv, kAdjTransmit, kGrad, kImGrad, kAccum, kDW, kDWExp, kRotShift,
    // UTR reconstruction
    kUtrImgRows, kUtrImgCols, kUtrGrid, kUtrFourier, kUtrVolCols, kUtrFinal, kUtrPoint,
    // the tilt series' image copy to host memory (event-timed, not a kernel)
    kCopyImages,
    // the whole slice loop of a small grid in one cluster launch
    kSmall,
    kKinds
};
extern const char *const kKindName[kKinds];

struct ProfRec {
    int kind;
    cudaEvent_t a, b;
    double bytes;
};

}  // namespace msk

struct msk_context {
    int device = 0;
    cudaStream_t stream = nullptr;      // the stream work goes to
    cudaStream_t own_stream = nullptr;  // created with the context
    cudaStream_t aux = nullptr;         // second stream: the wave chain of the slice loop,
                                        // the potential stacks' copies in
    cudaStream_t aux2 = nullptr;        // third stream: the potential stacks' copies out
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_t[2] = {}, ev_free[2] = {};
    bool prof_on = false;
    std::vector<msk::ProfRec> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    long long prof_launches[msk::kKinds] = {};
    double prof_ms[msk::kKinds] = {}, prof_bytes[msk::kKinds] = {};
    long long copies[2] = {};      // host-to-device, device-to-host copies while profiling
    double copy_bytes[2] = {};
    std::string err;
    msk::DevBuf psi, tbuf, tbuf2, atoms, slice_off, act, tables, imgmeta, wave0, images, exitw,
        fresnel, flags;
    msk::DevBuf pa_v, pa_t, pa_psi, pa_e;  // buffers of the per-orientation comparison form
    msk::DevBuf stk, stk_v, stk_g, stk_t, stk_img, stk_part, adjtab;  // potential stacks, adjoint
    msk::DevBuf arena;                                // specimen batches
    msk::DevBuf dwbuf;                                // Debye-Waller -B/4 per (unit, slice)
    msk::DevBuf imgfill;                              // image-plane fill values per unit
    msk::DevBuf tune;                                 // scratch grids of the schedule tuners
    msk::DevBuf utr_img, utr_k2, utr_acc, utr_vol, utr_out, utr_tab, utr_stage;  // UTR reconstruction
    bool no_tune = false;                             // schedules fixed at variant 0
    bool no_host_stage = false;                       // no page-locked staging (allocates none)
    void *h_stage = nullptr;                          // page-locked staging of a batch's atoms
    size_t h_stage_cap = 0;
    std::vector<float> w0_host;                       // msk_calculate's last incident wave,
    const void *w0_dev = nullptr;                     // uploaded to this wave0 buffer
    bool w0_valid = false;
    cudaEvent_t stk_ev[7] = {};                       // potential stacks: copy / kernel handoffs
    std::vector<cudaEvent_t> stk_sev;                 // the same per slice (2 per slice)
    std::vector<cudaStream_t> lanes;                  // concurrent specimens of a batch
    std::vector<cudaEvent_t> lane_ev;                 // lane joins (one per lane) + fork
    size_t units_alloc = 0;  // units the psi / tbuf buffers hold
    // msk_calculate's grid and tables as last uploaded (its grid parameters
    // and atomic numbers): repeated calls on one grid skip their preparation;
    // any other upload of the tables clears it
    std::shared_ptr<void> calc_cache;
    std::vector<int> zmap = std::vector<int>(104, -1);
};

namespace msk {

// Sets the context's error text; returns `code`.
int fail(msk_context *ctx, int code, const std::string &msg);

#define MSK_CUDA(ctx, call)                                                                     \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return msk::fail(ctx, e_ == cudaErrorMemoryAllocation ? MSK_ENOMEM : MSK_ECUDA,     \
                             std::string(#call) + ": " + cudaGetErrorString(e_));               \
    } while (0)

bool pow2_supported(int n);
// Stockham stage twiddles of the line FFT of length n (false: no kernels for n).
// ev = 16: the twiddles of the 16-points-a-thread plan FftPlan<n, 16>.
bool twiddles(int n, std::vector<float2> &out, int ev = 0);
bool is_device_ptr(const void *p);
bool is_pinned_host(const void *p);
// The device address of mapped page-locked host memory, or null.
void *mapped_host(void *p);

// cuTensorMapEncodeTiled through the runtime's driver entry point.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// 2D view of a buffer of `units` blocks of nx rows x ny complex64 for the
// column passes of tile variant v (box: the variant's column tile).
int column_map(msk_context *ctx, ColView *view, void *base, int nx, int ny, size_t units,
               const SizeOps *cop, int v);

// Device error flags: cleared at the start of a call, read after its last
// synchronisation (a bounded wait in a kernel that gave up sets a bit).
int flags_reset(msk_context *ctx, Geom &g);
int flags_check(msk_context *ctx);

// Host<->device copy accounting (dir 0: to the device, 1: to the host).
void count_copy(msk_context *ctx, int dir, double bytes);
// After a stream synchronisation: fold the recorded events into the totals.
void prof_collect(msk_context *ctx);

// Brackets one launch with events when profiling is on.
struct Prof {
    msk_context *ctx;
    int kind;
    double bytes;
    cudaEvent_t a = nullptr;
    static cudaEvent_t get(msk_context *c)
    {
        if (!c->prof_pool.empty()) {
            cudaEvent_t e = c->prof_pool.back();
            c->prof_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    cudaStream_t st;
    Prof(msk_context *c, int k, double b, cudaStream_t stream = nullptr)
        : ctx(c), kind(k), bytes(b), st(stream ? stream : c->stream)
    {
        if (ctx->prof_on) {
            a = get(ctx);
            cudaEventRecord(a, st);
        }
    }
    ~Prof()
    {
        if (a) {
            cudaEvent_t b = get(ctx);
            cudaEventRecord(b, st);
            ctx->prof_pending.push_back({kind, a, b, bytes});
        }
    }
};

}  // namespace msk
