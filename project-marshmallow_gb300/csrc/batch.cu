// batch.cu - many views of uneven size in one persistent launch (mm_clouds_march_batch).
//
// Every view becomes a launch record (the same MarchLaunch the single-view kernels take: uniform
// blocks, texture views, output image).  The work of all views is one queue of warp tiles (32 rays
// each, tw x 32/tw pixels), numbered view after view; persistent warps take chunks of `grab`
// consecutive tiles from one global counter, find the view by a binary search over the views'
// first-tile indices, read that view's record from constant memory and march the tile's rays
// exactly as march_tiled_kernel does; within a view the tile rows just above its horizon come first.  The record upload, the counter reset and the kernel are captured into
// a CUDA graph once per (view count, options, textures) and replayed for later batches.  The
// default schedule (MM_BATCH_BLOCKS) is one ordinary launch over 16x8-pixel blocks of all views
// instead: blocks of one SM then cover compact neighbouring tiles, as in march_tiled_kernel.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "march_kernel.cuh"

namespace mm {
namespace batch {

using namespace march;

constexpr int kWarps = 4;
constexpr int kMaxViews = 1024;
constexpr int kViewsPerLaunch = 72;  // launch records held in constant memory per launch

// The views of one launch live in constant memory: a warp reads its view's fields with a
// warp-uniform index, which the constant cache broadcasts like kernel parameters.
__constant__ MarchLaunch c_views[kViewsPerLaunch];
__constant__ int c_first_tile[kViewsPerLaunch + 1];

struct Queue {
    int n;
    int tw;                    // warp tile width (pixels); height = 32 / tw
    int grab;                  // tiles per queue access
    unsigned int* counter;
};

#ifndef MM_BATCH_MIN_BLOCKS
#define MM_BATCH_MIN_BLOCKS 9
#endif

__global__ void __launch_bounds__(kWarps * 32, MM_BATCH_MIN_BLOCKS) batch_kernel(Queue q) {
    __shared__ V3 s_cone[kWarps][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int total = c_first_tile[q.n];
    const int th = 32 / q.tw;
    int cur_view = -1;
    while (true) {
        int t0 = 0;
        if (lane == 0) t0 = (int)atomicAdd(q.counter, (unsigned)q.grab) ;
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= total) break;
        for (int tile = t0; tile < t0 + q.grab && tile < total; ++tile) {
            // view of this tile: last v with first_tile[v] <= tile
            int lo = 0, hi = q.n - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (c_first_tile[mid] <= tile) lo = mid; else hi = mid - 1;
            }
            const int v = lo;
            if (v != cur_view) {  // warp-uniform: the view's cone offsets
                __syncwarp();
                if (lane < 6) {
                    const float* b = c_views[v].u.sun.direction_basis;
                    float x, y, z;
                    switch (lane) {
                        case 0: x = 0.0f; y = 0.6f; z = 0.0f; break;
                        case 1: x = 0.0f; y = 0.5f; z = 0.05f; break;
                        case 2: x = 0.1f; y = 0.75f; z = 0.0f; break;
                        case 3: x = 0.2f; y = 2.5f; z = 0.3f; break;
                        case 4: x = 0.0f; y = 6.0f; z = 0.0f; break;
                        default: x = -0.1f; y = 1.0f; z = -0.2f; break;
                    }
                    s_cone[wid][lane] = {(b[0] * x + b[4] * y) + b[8] * z, (b[1] * x + b[5] * y) + b[9] * z,
                                         (b[2] * x + b[6] * y) + b[10] * z};
                }
                __syncwarp();
                cur_view = v;
            }
            const MarchLaunch& p = c_views[v];
            const int local = tile - c_first_tile[v];
            const int tiles_x = (p.width + q.tw - 1) / q.tw;
            // tile rows just above the view's horizon first (the long rays; see horizon_row_split)
            const int r = local / tiles_x;
            const int row = r < p.row_split ? p.row_split - 1 - r : r;
            const int px = (local % tiles_x) * q.tw + lane % q.tw;
            const int py = row * th + lane / q.tw;
            if (px < p.width && py < p.height) {
                const Frame f = make_frame<false>(p);
                Work w;
                march_pixel<false, MM_SAMPLER_HARDWARE>(p, f, s_cone[wid], px, py, w);
            }
        }
    }
}

// MM_BATCH_BLOCKS: one ordinary launch over the blocks of all views.  Block b belongs to the view v
// whose first-block index is the last one <= b (c_first_tile holds block counts in this mode); the
// block marches a 16x8-pixel tile of that view, its block rows ordered horizon-first, exactly as
// march_tiled_kernel does for a single view, and the hardware block scheduler balances the load.
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_MARCH_MIN_BLOCKS) batch_blocks_kernel(int n) {
    __shared__ V3 s_cone[6];
    const int b = (int)blockIdx.x;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (c_first_tile[mid] <= b) lo = mid; else hi = mid - 1;
    }
    const MarchLaunch& p = c_views[lo];
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const int local = b - c_first_tile[lo];
    const int blocks_x = (p.width + kBlockTileW - 1) / kBlockTileW;
    const int r = local / blocks_x;
    const int by = r < p.row_split ? p.row_split - 1 - r : r;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = tile_px(local % blocks_x, warp, lane);
    const int py = tile_py(by, warp, lane);
    if (px >= p.width || py >= p.height) return;
    const Frame f = make_frame<false>(p);
    Work w;
    march_pixel<false, MM_SAMPLER_HARDWARE>(p, f, s_cone, px, py, w);
}

}  // namespace batch
}  // namespace mm

// ------------------------------------------------------------------------------ host side

namespace {

struct BatchState {
    mm::MarchLaunch* h_views = nullptr;  // pinned staging
    int* h_first = nullptr;              // pinned staging
    mm::MarchLaunch* d_views = nullptr;
    int* d_first = nullptr;  // unused: records live in constant memory
    int cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;  // the last batch that read the staging buffers
    int g_n = -1, g_tw = 0, g_grab = 0, g_grid = 0, g_launches = 0, g_sched = -1;
    // MM_BATCH_GRAPH: capture streams (one per branch) and their fork/join events
    static constexpr int kBranches = 4;
    cudaStream_t branch[kBranches] = {};
    cudaEvent_t fork = nullptr, join[kBranches] = {};
};

// Views in order of decreasing ray count, dealt round-robin to the graph's branches (the longest
// launches start first on every branch; the small ones fill the others' tails).
int capture_views(mm_context ctx, BatchState* b, const mm_view* views, int n, const mm_scene_textures* tex,
                  const mm_batch_options& o, cudaGraph_t* out) {
    constexpr int K = BatchState::kBranches;
    if (!b->fork) {
        MM_CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        for (int k = 0; k < K; ++k) {
            MM_CUDA_TRY(cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking));
            MM_CUDA_TRY(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
        }
    }
    int* order = new (std::nothrow) int[n];
    if (!order) return mm::fail(MM_ERR_OUT_OF_MEMORY, "batch: host allocation");
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = 1; i < n; ++i) {  // insertion sort by decreasing pixel count (n <= 1024)
        const int v = order[i];
        const long long pv = (long long)views[v].out.width * views[v].out.height;
        int j = i - 1;
        while (j >= 0 && (long long)views[order[j]].out.width * views[order[j]].out.height < pv) {
            order[j + 1] = order[j];
            --j;
        }
        order[j + 1] = v;
    }
    int r = MM_OK;
    cudaError_t e = cudaStreamBeginCapture(b->branch[0], cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        delete[] order;
        return mm::cuda_fail(e, "batch graph capture");
    }
    cudaEventRecord(b->fork, b->branch[0]);
    for (int k = 1; k < K; ++k) cudaStreamWaitEvent(b->branch[k], b->fork, 0);
    for (int i = 0; i < n && r == MM_OK; ++i) {
        const mm_view& v = views[order[i]];
        mm_march_options mo;
        mm_march_options_default(&mo);
        mo.coverage_offset = v.coverage_offset;
        mo.density_format = o.density_format;
        mm::MarchLaunch p;
        mm::fill_march_launch(v.u, tex, v.out, mo, &p);
        // Surrogate views share the context's records: they run one after another on branch 0.  A
        // view with the sun below the horizon takes the plain cone, as a single march does.
        if (o.surrogate && v.u.sun.direction[1] >= 0.0f)
            r = mm::launch_surrogate_frame(p, ctx, o.surrogate, b->branch[0]);
        else
            r = mm::launch_march_fast(p, MM_SAMPLER_HARDWARE, o.density_format, MM_SCHEDULE_TILED, 0, ctx->d_work,
                                      ctx->num_sms, b->branch[o.surrogate ? 0 : i % K]);
    }
    for (int k = 1; k < K; ++k) {
        cudaEventRecord(b->join[k], b->branch[k]);
        cudaStreamWaitEvent(b->branch[0], b->join[k], 0);
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->branch[0], &g);
    delete[] order;
    if (r == MM_OK && e != cudaSuccess) r = mm::cuda_fail(e, "batch graph capture");
    if (r != MM_OK) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    *out = g;
    return MM_OK;
}

BatchState* state_of(mm_context ctx) { return reinterpret_cast<BatchState*>(ctx->batch); }

void drop_graph(BatchState* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->g_n = -1;
}

int ensure_capacity(BatchState* b, int n) {
    if (b->cap >= n) return MM_OK;
    drop_graph(b);
    cudaFreeHost(b->h_views);
    cudaFreeHost(b->h_first);
    cudaFree(b->d_views);
    cudaFree(b->d_first);
    b->h_views = nullptr;
    b->h_first = nullptr;
    b->d_views = nullptr;
    b->d_first = nullptr;
    b->cap = 0;
    const int groups = (n + mm::batch::kViewsPerLaunch - 1) / mm::batch::kViewsPerLaunch;
    MM_CUDA_TRY(cudaMallocHost(&b->h_views, n * sizeof(mm::MarchLaunch)));
    MM_CUDA_TRY(cudaMallocHost(&b->h_first, (size_t)groups * (mm::batch::kViewsPerLaunch + 1) * sizeof(int)));
    b->cap = n;
    return MM_OK;
}

// One launch per group of up to kViewsPerLaunch views: records to constant memory, counter reset,
// persistent kernel.  Returns the number of launches through *launches.
int enqueue(mm_context ctx, BatchState* b, int n, int tw, int grab, int grid, int sched, cudaStream_t s,
            int* launches) {
    using mm::batch::kViewsPerLaunch;
    *launches = 0;
    for (int v0 = 0; v0 < n; v0 += kViewsPerLaunch) {
        const int m = n - v0 < kViewsPerLaunch ? n - v0 : kViewsPerLaunch;
        int* first = b->h_first + (size_t)(v0 / kViewsPerLaunch) * (kViewsPerLaunch + 1);
        MM_CUDA_TRY(cudaMemcpyToSymbolAsync(mm::batch::c_views, b->h_views + v0, m * sizeof(mm::MarchLaunch), 0,
                                            cudaMemcpyHostToDevice, s));
        MM_CUDA_TRY(cudaMemcpyToSymbolAsync(mm::batch::c_first_tile, first, (m + 1) * sizeof(int), 0,
                                            cudaMemcpyHostToDevice, s));
        if (sched == MM_BATCH_BLOCKS) {
            mm::batch::batch_blocks_kernel<<<first[m], MM_TILED_WARPS * 32, 0, s>>>(m);
        } else {
            MM_CUDA_TRY(cudaMemsetAsync(ctx->d_work + 2, 0, sizeof(unsigned int), s));
            mm::batch::Queue q;
            q.n = m;
            q.tw = tw;
            q.grab = grab;
            q.counter = ctx->d_work + 2;
            mm::batch::batch_kernel<<<grid, mm::batch::kWarps * 32, 0, s>>>(q);
        }
        MM_CUDA_TRY(cudaGetLastError());
        ++*launches;
    }
    return MM_OK;
}

}  // namespace

namespace mm {
void batch_state_destroy(mm_context ctx) {
    BatchState* b = state_of(ctx);
    if (!b) return;
    drop_graph(b);
    if (b->done) cudaEventSynchronize(b->done);
    if (b->done) cudaEventDestroy(b->done);
    for (int k = 0; k < BatchState::kBranches; ++k) {
        if (b->branch[k]) cudaStreamDestroy(b->branch[k]);
        if (b->join[k]) cudaEventDestroy(b->join[k]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    cudaFreeHost(b->h_views);
    cudaFreeHost(b->h_first);
    cudaFree(b->d_views);
    cudaFree(b->d_first);
    delete b;
    ctx->batch = nullptr;
}
}  // namespace mm

extern "C" int mm_batch_options_default(mm_batch_options* o) {
    if (!o) return mm::fail(MM_ERR_INVALID_ARGUMENT, "batch options: null pointer");
    memset(o, 0, sizeof(*o));
    o->warp_tile_w = 8;
    o->tiles_per_grab = 4;
    o->use_graph = 1;
    o->schedule = MM_BATCH_GRAPH;
    return MM_OK;
}

extern "C" int mm_clouds_march_batch(mm_context ctx, const mm_view* views, int n, const mm_scene_textures* tex,
                                     const mm_batch_options* opt, void* stream) {
    using mm::fail;
    if (!ctx || !views || !tex || n <= 0) return fail(MM_ERR_INVALID_ARGUMENT, "batch: bad arguments");
    if (n > mm::batch::kMaxViews) return fail(MM_ERR_INVALID_ARGUMENT, "batch: more than %d views", mm::batch::kMaxViews);
    mm_batch_options o;
    if (opt)
        o = *opt;
    else
        mm_batch_options_default(&o);
    if (o.warp_tile_w != 4 && o.warp_tile_w != 8 && o.warp_tile_w != 16 && o.warp_tile_w != 32)
        return fail(MM_ERR_INVALID_ARGUMENT, "batch: warp_tile_w must be 4, 8, 16 or 32");
    if (o.tiles_per_grab < 1 || o.tiles_per_grab > 64)
        return fail(MM_ERR_INVALID_ARGUMENT, "batch: tiles_per_grab must be in [1, 64]");
    if (o.schedule != MM_BATCH_BLOCKS && o.schedule != MM_BATCH_PERSISTENT && o.schedule != MM_BATCH_GRAPH)
        return fail(MM_ERR_INVALID_ARGUMENT, "batch: bad schedule %d", o.schedule);
    if (o.surrogate && o.schedule != MM_BATCH_GRAPH)
        return fail(MM_ERR_INVALID_ARGUMENT, "batch: the surrogate cone needs the graph schedule");
    // Validate textures and images as a single-view march would, through its own checks.
    for (int i = 0; i < n; ++i) {
        mm_march_options mo;
        mm_march_options_default(&mo);
        mo.coverage_offset = views[i].coverage_offset;
        mo.density_format = o.density_format;
        if (o.surrogate) {
            mo.cone = MM_CONE_SURROGATE;
            mo.surrogate = o.surrogate;
        }
        int r = mm::validate_march(ctx, &views[i].u, tex, &views[i].out, &mo);
        if (r) {
            char msg[400];
            snprintf(msg, sizeof(msg), "%s", mm_last_error_string());
            return fail(r, "batch: view %d: %s", i, msg);
        }
    }
    if (!ctx->batch) {
        ctx->batch = new (std::nothrow) BatchState;
        if (!ctx->batch) return fail(MM_ERR_OUT_OF_MEMORY, "batch: host allocation");
    }
    BatchState* b = state_of(ctx);
    if (!b->done) MM_CUDA_TRY(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    // The previous batch's upload reads the pinned staging buffers: let it finish first.
    MM_CUDA_TRY(cudaEventSynchronize(b->done));
    if (o.schedule == MM_BATCH_GRAPH) {
        // Each view's own launch (its kernel variant, uniforms by value) captured on the branches,
        // then applied to the executable graph (cudaGraphExecUpdate) or instantiated anew.
        cudaGraph_t g = nullptr;
        if (o.surrogate) {  // the deferred-sample records of the largest view, allocated before the capture
            size_t most = 0;
            for (int i = 0; i < n; ++i) {
                const size_t px = (size_t)views[i].out.width * views[i].out.height;
                if (px > most) most = px;
            }
            int rr = mm::surrogate_reserve(ctx, most);
            if (rr) return rr;
        }
        int r = capture_views(ctx, b, views, n, tex, o, &g);
        if (r) return r;
        bool updated = false;
        if (b->exec && b->g_sched == MM_BATCH_GRAPH && b->g_n == n) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(b->exec, g, &info) == cudaSuccess;
            if (!updated) cudaGetLastError();  // clear the update failure; instantiate below
        }
        if (updated) {
            cudaGraphDestroy(g);
        } else {
            drop_graph(b);
            b->graph = g;
            cudaError_t e = cudaGraphInstantiate(&b->exec, g, 0);
            if (e != cudaSuccess) {
                drop_graph(b);
                return mm::cuda_fail(e, "batch graph instantiate");
            }
            b->g_n = n;
            b->g_sched = MM_BATCH_GRAPH;
        }
        MM_CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
        mm::count_launch(n);
        MM_CUDA_TRY(cudaEventRecord(b->done, (cudaStream_t)stream));
        return MM_OK;
    }
    int r = ensure_capacity(b, n);
    if (r) return r;
    const int th = 32 / o.warp_tile_w;
    const int K = mm::batch::kViewsPerLaunch;
    for (int v0 = 0; v0 < n; v0 += K) {  // tile numbering restarts in every launch group
        int* first = b->h_first + (size_t)(v0 / K) * (K + 1);
        int total = 0, i = v0;
        for (; i < n && i < v0 + K; ++i) {
            mm_march_options mo;
            mm_march_options_default(&mo);
            mo.coverage_offset = views[i].coverage_offset;
            mm::fill_march_launch(views[i].u, tex, views[i].out, mo, &b->h_views[i]);
            // units of the queue: 16x8-pixel blocks (MM_BATCH_BLOCKS) or warp tiles of tw x th pixels
            const int uw = o.schedule == MM_BATCH_BLOCKS ? mm::march::kBlockTileW : o.warp_tile_w;
            const int uh = o.schedule == MM_BATCH_BLOCKS ? mm::march::kBlockTileH : th;
            const int unit_rows = (views[i].out.height + uh - 1) / uh;
            b->h_views[i].row_split = mm::march::horizon_row_split(b->h_views[i], unit_rows, uh);
            first[i - v0] = total;
            total += ((views[i].out.width + uw - 1) / uw) * unit_rows;
        }
        first[i - v0] = total;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mm::batch::batch_kernel, mm::batch::kWarps * 32, 0);
    if (per_sm < 1) per_sm = 1;
    const int grid = ctx->num_sms * per_sm;
    cudaStream_t s = (cudaStream_t)stream;
    int launches = 0;
    if (!o.use_graph) {
        r = enqueue(ctx, b, n, o.warp_tile_w, o.tiles_per_grab, grid, o.schedule, s, &launches);
        if (!r) mm::count_launch(launches);
        if (!r) MM_CUDA_TRY(cudaEventRecord(b->done, s));
        return r;
    }
    if (!b->exec || b->g_n != n || b->g_tw != o.warp_tile_w || b->g_grab != o.tiles_per_grab || b->g_grid != grid ||
        b->g_sched != o.schedule) {
        drop_graph(b);
        cudaStream_t cap_stream;
        MM_CUDA_TRY(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            r = enqueue(ctx, b, n, o.warp_tile_w, o.tiles_per_grab, grid, o.schedule, cap_stream, &launches);
            cudaGraph_t g = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(cap_stream, &g);
            if (r == MM_OK && e2 != cudaSuccess) r = mm::cuda_fail(e2, "batch graph capture");
            if (r == MM_OK) {
                b->graph = g;
                e2 = cudaGraphInstantiate(&b->exec, g, 0);
                if (e2 != cudaSuccess) r = mm::cuda_fail(e2, "batch graph instantiate");
            } else if (g) {
                cudaGraphDestroy(g);
            }
        } else {
            r = mm::cuda_fail(e, "batch graph capture");
        }
        cudaStreamDestroy(cap_stream);
        if (r) {
            drop_graph(b);
            return r;
        }
        b->g_n = n;
        b->g_tw = o.warp_tile_w;
        b->g_grab = o.tiles_per_grab;
        b->g_grid = grid;
        b->g_sched = o.schedule;
        b->g_launches = launches;
    }
    // The graph copies the pinned staging buffers, which hold this batch's records now.
    MM_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    mm::count_launch(b->g_launches);
    MM_CUDA_TRY(cudaEventRecord(b->done, s));
    return MM_OK;
}

// Times every (warp tile width, tiles per grab) pair of the persistent schedule, the block schedule
// and the graph schedule on the given batch and returns the fastest.
extern "C" int mm_batch_autotune(mm_context ctx, const mm_view* views, int n, const mm_scene_textures* tex,
                                 mm_batch_options* best, float* ms_table, void* stream) {
    if (!best) return mm::fail(MM_ERR_INVALID_ARGUMENT, "autotune: null result");
    const int tws[4] = {4, 8, 16, 32}, grabs[5] = {1, 2, 4, 8, 16};
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    MM_CUDA_TRY(cudaEventCreate(&e0));
    MM_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 3.4e38f;
    int r = MM_OK;
    for (int a = 0; a < 6 && r == MM_OK; ++a)
        for (int g = 0; g < (a < 4 ? 5 : 1) && r == MM_OK; ++g) {
            mm_batch_options o;
            mm_batch_options_default(&o);
            if (a < 4) {
                o.schedule = MM_BATCH_PERSISTENT;
                o.warp_tile_w = tws[a];
                o.tiles_per_grab = grabs[g];
            } else {
                o.schedule = a == 4 ? MM_BATCH_BLOCKS : MM_BATCH_GRAPH;
            }
            if ((r = mm_clouds_march_batch(ctx, views, n, tex, &o, stream))) break;  // warm-up and capture
            cudaEventRecord(e0, s);
            if ((r = mm_clouds_march_batch(ctx, views, n, tex, &o, stream))) break;
            cudaEventRecord(e1, s);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                r = mm::cuda_fail(e, "autotune");
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms_table) ms_table[a < 4 ? a * 5 + g : 20 + (a - 4)] = ms;
            if (ms < best_ms) {
                best_ms = ms;
                *best = o;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return r;
}
