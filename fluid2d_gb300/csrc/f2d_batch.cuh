// f2d_batch.cuh -- one launch per kernel for many independent instances.
//
// Every engine kernel is a body `run(args, vb)` that reads its block
// coordinates from a VB (virtual block) instead of blockIdx/gridDim.  A
// native launch passes the real coordinates; a batched launch covers the
// blocks of many instances in one grid: a block finds its instance in the
// prefix sums of the instances' block counts and runs the body with that
// instance's arguments and local coordinates.  The arithmetic is the same
// code, so an instance evolves bit for bit as it does alone.
//
// Batched steps are built by recording: while a Recorder is installed on the
// host thread, the launchers append (body kind, arguments, grid, block,
// shared memory) to it instead of launching (batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <type_traits>

#include "f2d_common.cuh"

namespace f2d {

struct VB {
    int x, y, gx, gy;
};

// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialisation attribute may be set up while its predecessor in the
// stream finishes; it waits here until that predecessor has completed and
// its memory is visible, so nothing it reads can be stale.  No kernel
// triggers its dependents early (an early trigger let the next kernel's
// blocks sit on SM resources beside a running kernel): the implicit trigger
// as each block exits overlaps only the launch of the next kernel with the
// tail of this one.
F2D_DEV void pdl_prologue() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// whether the launchers below use programmatic dependent launch (default on:
// 2-4 % shorter 1024^2 float64 and mixed steps, 1.5 % on the batched ensemble)
bool &pdl_enabled();

// The L2 access-policy window the launches of this host thread carry (a
// persisting window over a multigrid hierarchy's small levels, set by the
// hierarchy around its cycles; num_bytes 0: none)
cudaAccessPolicyWindow &l2_window();

template <typename A>
int launch_pdl(void (*kernel)(A), const A &a, dim3 grid, dim3 block, size_t smem,
               cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    int n = 0;
    if (pdl_enabled()) {
        attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[n].val.programmaticStreamSerializationAllowed = 1;
        n++;
    }
    const cudaAccessPolicyWindow &w = l2_window();
    if (w.num_bytes) {
        attr[n].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[n].val.accessPolicyWindow = w;
        n++;
    }
    cfg.attrs = attr;
    cfg.numAttrs = n;
    return (int)cudaLaunchKernelEx(&cfg, kernel, a);
}
#define F2D_VB_NATIVE \
    (VB{(int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x, (int)gridDim.y})

// the block -> instance map of a batched launch
struct BatchGrid {
    const int *start;  // [n + 1] first block of each instance
    const int *gxy;    // [2n] the instance's grid (x, y)
    int n;
};

F2D_DEV int batch_instance(const BatchGrid &g, int b) {
    int lo = 0, hi = g.n - 1;  // the last i with start[i] <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g.start[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// a Body may ask for a minimum of resident CTAs per SM (MIN_BLOCKS), which
// caps its registers as in its native kernel
template <class B, class = void>
struct body_min_blocks {
    static constexpr int value = 1;
};
template <class B>
struct body_min_blocks<B, std::void_t<decltype(B::MIN_BLOCKS)>> {
    static constexpr int value = B::MIN_BLOCKS;
};

template <class Body>
__global__ void __launch_bounds__(Body::THREADS, body_min_blocks<Body>::value)
    k_batch(const typename Body::Args *args, BatchGrid g) {
    using Args = typename Body::Args;
    static_assert(sizeof(Args) % 4 == 0, "argument blocks are copied as words");
    // the instance's arguments go to shared memory once per block: the body
    // then reads them from there as it needs them instead of holding them in
    // registers (as a kernel's own parameters are held in constant memory)
    __shared__ __align__(16) unsigned char abuf[sizeof(Args)];
    pdl_prologue();
    const int i = batch_instance(g, (int)blockIdx.x);
    const int nthr = (int)(blockDim.x * blockDim.y);
    const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
    for (int w = tid; w < (int)(sizeof(Args) / 4); w += nthr)
        ((int *)abuf)[w] = ((const int *)(args + i))[w];
    __syncthreads();
    const int lb = (int)blockIdx.x - g.start[i];
    const int gx = g.gxy[2 * i];
    Body::run(*(const Args *)abuf, VB{lb % gx, lb / gx, gx, g.gxy[2 * i + 1]});
}

// body kinds (the registry in batch.cu maps each to its batched launcher)
#define F2D_BODY_KINDS(X)                                                                      \
    X(SetDt) X(SplitF32) X(ToF32) X(AdvMixed) X(C2CF32) X(ResidualMixed) X(AddF32)           \
    X(OrthoMixed) X(Banom) X(CellToCorner) X(Reduce8P) X(Reduce8F) X(Reduce2P) X(Reduce2F)  \
    X(SolveInit) X(SolveUpdate) X(DiagP) X(DiagF) X(StageAdv64) X(StageOrtho) X(VecAdd)     \
    X(SubMean) X(Sweep1D1) X(Sweep2D1) X(ResidualD1) X(RestrictD) X(RestrictF) X(InterpD)   \
    X(SmoothFusedD0) X(SmoothFusedF0) X(SmoothFusedF1) X(ResresD0) X(ResresF0) X(ResresF1) \
    X(CoarseD) X(CoarseF) X(CoarseApplyD) X(CoarseApplyF)

enum BodyKind {
#define F2D_KIND_ENUM(n) BK_##n,
    F2D_BODY_KINDS(F2D_KIND_ENUM)
#undef F2D_KIND_ENUM
        BK_COUNT
};

using BatchLaunchFn = int (*)(const void *args, const BatchGrid &g, unsigned blocks, dim3 block,
                              size_t smem, cudaStream_t s);

#define F2D_KIND_DECL(n)                                                                   \
    int batch_launch_##n(const void *args, const BatchGrid &g, unsigned blocks, dim3 block, \
                         size_t smem, cudaStream_t s);
F2D_BODY_KINDS(F2D_KIND_DECL)
#undef F2D_KIND_DECL

// defines batch_launch_<kind> for a Body (in the translation unit of its body)
#define F2D_BATCH_ENTRY(n, Body)                                                              \
    int batch_launch_##n(const void *args, const BatchGrid &g, unsigned blocks, dim3 block,    \
                         size_t smem, cudaStream_t s) {                                        \
        cudaLaunchConfig_t cfg = {};                                                          \
        cfg.gridDim = dim3(blocks);                                                           \
        cfg.blockDim = block;                                                                 \
        cfg.dynamicSmemBytes = smem;                                                          \
        cfg.stream = s;                                                                       \
        cudaLaunchAttribute attr[1];                                                          \
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;                      \
        attr[0].val.programmaticStreamSerializationAllowed = 1;                               \
        cfg.attrs = attr;                                                                     \
        cfg.numAttrs = pdl_enabled() ? 1 : 0;                                                 \
        const typename Body::Args *a = (const typename Body::Args *)args;                     \
        cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch<Body>, a, g);                         \
        return cuda_status(e, "batched " #n);                                                 \
    }

struct Recorder {
    virtual int add(int kind, const void *args, size_t bytes, dim3 grid, dim3 block,
                    size_t smem) = 0;
    virtual ~Recorder() {}
};
// the recorder installed on this host thread (null: launch normally)
Recorder *&recorder();

// launch a body natively, or record it
template <class Body>
int launch_body(void (*native)(typename Body::Args), const typename Body::Args &a, dim3 grid,
                dim3 block, size_t smem, cudaStream_t s, const char *name) {
    if (Recorder *r = recorder()) return r->add(Body::KIND, &a, sizeof(a), grid, block, smem);
    return cuda_status((cudaError_t)launch_pdl(native, a, grid, block, smem, s), name);
}

}  // namespace f2d
