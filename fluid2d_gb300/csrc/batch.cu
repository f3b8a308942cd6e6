// batch.cu -- batched launches of many instances' steps.
//
// A step of every instance is recorded (the launchers append their body kind
// and arguments to a trace instead of launching), then the traces are merged
// into launches that each run one body for many instances: at every round
// the body that the most instances have next is launched for all of them,
// and those instances advance by one operation.  Each instance's operations
// keep their order and instances share no data, so every instance computes
// exactly what its own step computes.  The merged launches' arguments and
// block maps live in one device buffer; the launch sequence is captured once
// in a CUDA graph and replayed per step.
#include <algorithm>
#include <cstring>
#include <vector>

#include "f2d_batch.cuh"
#include "f2d_common.cuh"
#include "../../include/fluid2d_gb300.h"

namespace f2d {

#define BTRY(x)                 \
    do {                        \
        int _st = (x);          \
        if (_st) return _st;    \
    } while (0)

Recorder *&recorder() {
    static thread_local Recorder *r = nullptr;
    return r;
}

bool &pdl_enabled() {
    static bool on = true;
    return on;
}

cudaAccessPolicyWindow &l2_window() {
    static thread_local cudaAccessPolicyWindow w = {};
    return w;
}

static BatchLaunchFn batch_launcher(int kind) {
    static const BatchLaunchFn table[BK_COUNT] = {
#define F2D_KIND_FN(n) &batch_launch_##n,
        F2D_BODY_KINDS(F2D_KIND_FN)
#undef F2D_KIND_FN
    };
    return (kind >= 0 && kind < BK_COUNT) ? table[kind] : nullptr;
}

struct BatchOp {
    int kind;
    std::vector<unsigned char> args;
    dim3 grid, block;
    size_t smem;
};

struct TraceRecorder : Recorder {
    std::vector<BatchOp> ops;
    int add(int kind, const void *args, size_t bytes, dim3 grid, dim3 block,
            size_t smem) override {
        if (kind < 0 || kind >= BK_COUNT) {
            set_error("batch: a step operation has no batched form");
            return ERR_ARG;
        }
        BatchOp op;
        op.kind = kind;
        op.args.assign((const unsigned char *)args, (const unsigned char *)args + bytes);
        op.grid = grid;
        op.block = block;
        op.smem = smem;
        ops.push_back(op);
        return OK;
    }
};

struct BatchLaunch {
    int kind, n;
    size_t o_args, o_start, o_gxy;
    unsigned blocks;
    dim3 block;
    size_t smem;
};

struct BatchPlan {
    std::vector<BatchLaunch> launches;
    char *dev = nullptr;
    size_t bytes = 0;
    size_t ops = 0;
    ~BatchPlan() {
        if (dev) cudaFree(dev);
    }
    int run(cudaStream_t s) const {
        for (const BatchLaunch &L : launches) {
            BatchGrid g{(const int *)(dev + L.o_start), (const int *)(dev + L.o_gxy), L.n};
            BatchLaunchFn fn = batch_launcher(L.kind);
            int st = fn(dev + L.o_args, g, L.blocks, L.block, L.smem, s);
            if (st) return st;
        }
        return OK;
    }
};

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

static bool same_block(const dim3 &a, const dim3 &b) {
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

// Merge the traces and upload.  policy 0: launch the body that the most
// instances have next; policy 1: launch the next body of the instance with
// the most operations left (the critical path), joined by every instance
// whose next operation is the same body.
static int plan_build(const std::vector<std::vector<BatchOp>> &traces, BatchPlan &plan,
                      int policy) {
    const int n = (int)traces.size();
    std::vector<size_t> next(n, 0);
    std::vector<unsigned char> host;
    auto put = [&](const void *p, size_t b) {
        size_t o = align_up(host.size());
        host.resize(o + b);
        memcpy(host.data() + o, p, b);
        return o;
    };
    for (const auto &t : traces) plan.ops += t.size();
    while (true) {
        int count[BK_COUNT] = {0};
        bool left = false;
        for (int i = 0; i < n; i++)
            if (next[i] < traces[i].size()) {
                count[traces[i][next[i]].kind]++;
                left = true;
            }
        if (!left) break;
        int kind = 0;
        if (policy == 1) {
            size_t most = 0;
            for (int i = 0; i < n; i++) {
                const size_t left_i = traces[i].size() - next[i];
                if (left_i > most) {
                    most = left_i;
                    kind = traces[i][next[i]].kind;
                }
            }
        } else {
            for (int k = 1; k < BK_COUNT; k++)
                if (count[k] > count[kind]) kind = k;
        }
        // instances whose next operation is this body, grouped by block shape
        std::vector<int> members;
        for (int i = 0; i < n; i++)
            if (next[i] < traces[i].size() && traces[i][next[i]].kind == kind) members.push_back(i);
        while (!members.empty()) {
            const dim3 blk = traces[members[0]][next[members[0]]].block;
            std::vector<int> grp, rest;
            for (int i : members)
                (same_block(traces[i][next[i]].block, blk) ? grp : rest).push_back(i);
            std::vector<unsigned char> args;
            std::vector<int> start(1, 0), gxy;
            size_t smem = 0;
            for (int i : grp) {
                const BatchOp &op = traces[i][next[i]];
                args.insert(args.end(), op.args.begin(), op.args.end());
                const long long b = (long long)op.grid.x * op.grid.y;
                if (op.grid.z != 1 || start.back() + b > 0x7fffffffLL) {
                    set_error("batch: grid too large to merge");
                    return ERR_LIMIT;
                }
                start.push_back(start.back() + (int)b);
                gxy.push_back((int)op.grid.x);
                gxy.push_back((int)op.grid.y);
                smem = std::max(smem, op.smem);
                next[i]++;
            }
            BatchLaunch L;
            L.kind = kind;
            L.n = (int)grp.size();
            L.o_args = put(args.data(), args.size());
            L.o_start = put(start.data(), start.size() * sizeof(int));
            L.o_gxy = put(gxy.data(), gxy.size() * sizeof(int));
            L.blocks = (unsigned)start.back();
            L.block = blk;
            L.smem = smem;
            if (L.blocks > 0) plan.launches.push_back(L);
            members = rest;
        }
    }
    plan.bytes = host.size() ? host.size() : 256;
    BTRY(cuda_status(cudaMalloc((void **)&plan.dev, plan.bytes), "batch cudaMalloc"));
    return cuda_status(cudaMemcpy(plan.dev, host.data(), host.size(), cudaMemcpyHostToDevice),
                       "batch upload");
}

int configure_batched_coarse();

// A batch: the plan and its captured graph.
struct Batch {
    BatchPlan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~Batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

// record one step per instance with `step_fn(i)`, merge, upload, capture
int batch_create(int n, int (*step_fn)(void *ctx, int i), void *ctx, int policy, void **out) {
    std::vector<std::vector<BatchOp>> traces(n);
    for (int i = 0; i < n; i++) {
        TraceRecorder rec;
        recorder() = &rec;
        int st = step_fn(ctx, i);
        recorder() = nullptr;
        if (st) return st;
        traces[i] = std::move(rec.ops);
    }
    Batch *B = new (std::nothrow) Batch();
    if (!B) return ERR_CUDA;
    int st = plan_build(traces, B->plan, policy);
    if (!st) st = configure_batched_coarse();
    cudaStream_t cs = nullptr;
    if (!st) st = cuda_status(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "batch stream");
    if (!st) {
        st = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal),
                         "batch capture");
        if (!st) {
            int st1 = B->plan.run(cs);
            int st2 = cuda_status(cudaStreamEndCapture(cs, &B->graph), "batch capture end");
            st = st1 ? st1 : st2;
        }
        if (!st) st = cuda_status(cudaGraphInstantiate(&B->exec, B->graph, 0), "batch instantiate");
        cudaStreamDestroy(cs);
    }
    if (st) {
        delete B;
        return st;
    }
    *out = B;
    return OK;
}

int batch_step(void *b, int nsteps, cudaStream_t s) {
    Batch *B = (Batch *)b;
    for (int k = 0; k < nsteps; k++)
        BTRY(cuda_status(cudaGraphLaunch(B->exec, s), "batch graph launch"));
    return OK;
}

int batch_info(void *b, int *launches, int *ops) {
    Batch *B = (Batch *)b;
    if (launches) *launches = (int)B->plan.launches.size();
    if (ops) *ops = (int)B->plan.ops;
    return OK;
}

void batch_destroy(void *b) { delete (Batch *)b; }

}  // namespace f2d

extern "C" {

// programmatic dependent launch of the engine kernels: on (1, the default) or
// off (0); returns the previous setting.  Graphs captured before a change
// keep the launches they were captured with.
int f2d_set_pdl(int enable) {
    const int prev = f2d::pdl_enabled() ? 1 : 0;
    if (enable >= 0) f2d::pdl_enabled() = enable != 0;
    return prev;
}

}  // extern "C"
