// batch.cu — registration of many image pairs at once (a perfusion series
// against its reference frame, a cohort of 3D pairs; src/2dmyoset-all2one-
// nonrigid.cc:124-190, src/3dmany2one-nonrigid.cc:118-187 run one
// registration per pair in parallel host threads).
//
// All pairs advance in lock step.  One step evaluates the cost+gradient of
// every unfinished pair at the point its minimizer proposes:
//   k_min_propose  (blocks x pairs) the minimizer's next evaluation point
//                  (and, in 3D, its float copy that the warp kernel reads)
//   warp, adjoint, gather of the split path over a work list of
//                  (pair, tile) / (pair, block) items covering all pairs
//   k_min_update   (blocks x pairs) the minimizer's decision
// The minimizers (GSL steepest descent as CGSLFDFMinimizer drives it,
// mia/core/minimizer/gsl.cc:122-156, and CGDSQMinimizer::do_run,
// mia/core/minimizer/gdsq.cc:60-122) are state machines in device memory, so
// a run of steps needs no host round trip and is captured once per level and
// pass as a CUDA graph that is relaunched until every pair has finished.
// Level transitions (scale filter, upscale, refine) follow
// TNonrigidRegisterImpl::run (mia/template/nonrigidregister.cxx:193-296).
#include <array>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mgr.h"
#include "driver.hh"
#include "level.hh"
#include "pyramid.hh"
#include "trace.hh"

namespace mgr {

void set_last_error(const std::string &msg);

namespace {

constexpr int MT = 256;

struct MinState {
    double f;       // cost at x
    double step;
    double f_old;   // gdsq
    double gnorm;   // gsl: |g|, set when g is
    int iter;
    int phase;      // 0: evaluate x0, 1: iterate
    int failed;     // gsl: a trial failed in this iteration
    int trials;     // gsl: trials in this iteration
    int done;
    int evals;
    int success;    // gdsq stop flags
    int status;     // 0 running/converged, 1 no progress, 2 max iterations
};

struct PairVec {
    double *x, *g, *xt, *gt;
    const double *costs;   // {image, penalty} at xt
    int n;
    float *xf;             // 3D: the level's float copy of xt (written with xt), else null
};

// The minimizer kernels spread each pair's vectors over blocks of MCH
// elements (grid: blocks x pairs).  Every block decides from the pair's
// state as it was at launch; the block that finishes last (per-pair
// counter) adds the blocks' partial sums in block order and is the only
// writer of the state, so the decision does not depend on block timing.
constexpr int MCH = 2048;

struct MinScratch {
    double *part;     // pairs x nblk x 3: per block sum, sum, max
    unsigned *count;  // pairs: blocks done
    int *moved;       // pairs: gsl trial point differs from x
    int nblk;
};

// sums of a and b and the maximum of c over the block, returned to every
// thread (fixed order)
__device__ void block_reduce3(double &a, double &b, double &c, double *red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
    __syncthreads();   // red may still be read by a previous call
    if (lane == 0) {
        red[w] = a;
        red[MT / 32 + w] = b;
        red[2 * MT / 32 + w] = c;
    }
    __syncthreads();
    a = 0.0;
    b = 0.0;
    c = 0.0;
    for (int k = 0; k < MT / 32; ++k) {
        a += red[k];
        b += red[MT / 32 + k];
        c = fmax(c, red[2 * MT / 32 + k]);
    }
}

// store this block's partials; true in the pair's last block, which then
// holds the totals (partials added in block order) in a, b, c
__device__ bool pair_totals(const MinScratch &m, int p, int nb, double &a, double &b, double &c, double *red)
{
    __shared__ bool last;
    block_reduce3(a, b, c, red);
    if (threadIdx.x == 0) {
        double *pp = m.part + (size_t(p) * m.nblk + blockIdx.x) * 3;
        pp[0] = a;
        pp[1] = b;
        pp[2] = c;
        __threadfence();
        last = atomicAdd(&m.count[p], 1u) == unsigned(nb - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    a = 0.0;
    b = 0.0;
    c = 0.0;
    for (int k = threadIdx.x; k < nb; k += MT) {
        const double *pp = m.part + (size_t(p) * m.nblk + k) * 3;
        a += __ldcg(pp);
        b += __ldcg(pp + 1);
        c = fmax(c, __ldcg(pp + 2));
    }
    block_reduce3(a, b, c, red);
    if (threadIdx.x == 0) m.count[p] = 0;
    return true;
}

__global__ void __launch_bounds__(MT) k_min_propose(MinState *st, const PairVec *vec, mgr_minimizer_desc mz,
                                                    int *active, MinScratch m)
{
    __shared__ double red[3 * MT / 32];
    const int p = blockIdx.y, tid = threadIdx.x;
    const PairVec v = vec[p];
    const int nb = (v.n + MCH - 1) / MCH;
    if (int(blockIdx.x) >= nb) return;
    const int i0 = blockIdx.x * MCH, i1 = min(v.n, i0 + MCH);
    const bool lead = blockIdx.x == 0 && tid == 0;
    const MinState s = st[p];
    if (s.done) {
        if (lead) active[p] = 0;
        return;
    }
    if (s.phase == 0) {
        for (int i = i0 + tid; i < i1; i += MT) {
            const double xi = v.x[i];
            v.xt[i] = xi;
            if (v.xf) v.xf[i] = float(xi);
        }
        if (lead) active[p] = 1;
        return;
    }
    if (mz.kind == MGR_MIN_GSL_SD) {
        if (s.gnorm == 0.0 || s.trials >= 2000) {
            if (lead) {
                st[p].done = 1;
                st[p].status = 1;
                active[p] = 0;
            }
            return;
        }
        const double a = -s.step / s.gnorm;
        int mv = 0;
        for (int i = i0 + tid; i < i1; i += MT) {
            const double x1 = __dadd_rn(v.x[i], __dmul_rn(a, v.g[i]));
            v.xt[i] = x1;
            if (v.xf) v.xf[i] = float(x1);
            if (x1 != v.x[i]) mv = 1;
        }
        mv = __syncthreads_or(mv);
        if (tid == 0 && mv) atomicOr(&m.moved[p], 1);
        double d0 = 0.0, d1 = 0.0, d2 = 0.0;
        if (!pair_totals(m, p, nb, d0, d1, d2, red)) return;
        if (tid == 0) {
            if (atomicExch(&m.moved[p], 0) == 0) {   // the step no longer changes x
                st[p].done = 1;
                st[p].status = 1;
                active[p] = 0;
            } else {
                st[p].trials = s.trials + 1;
                active[p] = 1;
            }
        }
    } else {
        // while (iter++ < maxiter && step > min_step && !success)
        const bool go = (s.iter < mz.maxiter) && (s.step > mz.min_step) && !s.success;
        if (!go) {
            if (lead) {
                st[p].iter = s.iter + 1;
                st[p].done = 1;
                active[p] = 0;
            }
            return;
        }
        const double ms = -s.step;
        for (int i = i0 + tid; i < i1; i += MT) {
            const double xi = __dadd_rn(v.xt[i], __dmul_rn(ms, v.g[i]));
            v.xt[i] = xi;
            if (v.xf) v.xf[i] = float(xi);
        }
        double d0 = 0.0, d1 = 0.0, d2 = 0.0;
        if (!pair_totals(m, p, nb, d0, d1, d2, red)) return;
        if (tid == 0) {
            st[p].iter = s.iter + 1;
            active[p] = 1;
        }
    }
}

__global__ void __launch_bounds__(MT) k_min_update(MinState *st, const PairVec *vec, mgr_minimizer_desc mz,
                                                   const int *active, MinScratch m)
{
    __shared__ double red[3 * MT / 32];
    const int p = blockIdx.y, tid = threadIdx.x;
    if (!active[p]) return;
    const PairVec v = vec[p];
    const int nb = (v.n + MCH - 1) / MCH;
    if (int(blockIdx.x) >= nb) return;
    const int i0 = blockIdx.x * MCH, i1 = min(v.n, i0 + MCH);
    const MinState s = st[p];
    const double fe = v.costs[0] + v.costs[1];
    double q = 0.0, q2 = 0.0, mx = 0.0;
    if (s.phase == 0) {
        for (int i = i0 + tid; i < i1; i += MT) {
            const double gi = v.gt[i];
            v.g[i] = gi;
            q += gi * gi;
            mx = fmax(mx, fabs(gi));
        }
        if (!pair_totals(m, p, nb, q, q2, mx, red)) return;
        if (tid == 0) {
            MinState &o = st[p];
            o.f = fe;
            o.f_old = fe;
            o.gnorm = sqrt(q);
            o.phase = 1;
            o.evals = s.evals + 1;
            // all |g| < xtol
            if (mz.kind == MGR_MIN_GDSQ && !(mx >= mz.xtol)) o.success = s.success | 1;
        }
        return;
    }
    if (mz.kind == MGR_MIN_GSL_SD) {
        if (fe > s.f) {
            if (blockIdx.x == 0 && tid == 0) {
                st[p].evals = s.evals + 1;
                st[p].failed = 1;
                st[p].step = s.step * mz.tol;
            }
            return;
        }
        for (int i = i0 + tid; i < i1; i += MT) {
            const double gi = v.gt[i];
            v.x[i] = v.xt[i];
            v.g[i] = gi;
            q += gi * gi;
        }
        if (!pair_totals(m, p, nb, q, q2, mx, red)) return;
        if (tid == 0) {
            MinState &o = st[p];
            const double gn = sqrt(q);
            o.gnorm = gn;
            o.evals = s.evals + 1;
            o.step = s.step * (s.failed ? mz.tol : 2.0);
            o.f = fe;
            o.failed = 0;
            o.trials = 0;
            o.iter = s.iter + 1;
            if (gn < mz.eps) o.done = 1;
            else if (o.iter >= mz.maxiter) {
                o.done = 1;
                o.status = 2;
            }
        }
        return;
    }
    // gdsq
    if (fe < s.f_old) {
        const double ms = -s.step;
        for (int i = i0 + tid; i < i1; i += MT) {
            const double gs = __dmul_rn(v.g[i], ms), gi = v.gt[i];
            q += gs * gi;
            q2 += gs * gs;
            v.x[i] = v.xt[i];
            v.g[i] = gi;
            mx = fmax(mx, fabs(gi));
        }
        if (!pair_totals(m, p, nb, q, q2, mx, red)) return;
        if (tid == 0) {
            MinState &o = st[p];
            const double nrm = sqrt(q2);
            double step = s.step;
            const double aux = s.f_old - fe + q;
            if (aux <= 0.0) step *= mz.scale;
            else step = 0.5 * nrm / aux;
            int success = s.success;
            if (!(mx >= mz.gtol)) success |= 2;        // all |g| < gtol
            if (s.f_old - fe < mz.ftolr) success |= 4;
            if (!(mx >= mz.xtol / step)) success |= 1;  // all |g| < xtol / step
            o.f_old = fe;
            o.f = fe;
            o.step = step;
            o.evals = s.evals + 1;
            o.success = success;
        }
    } else {
        for (int i = i0 + tid; i < i1; i += MT) {
            v.xt[i] = v.x[i];
            mx = fmax(mx, fabs(v.g[i]));
        }
        if (!pair_totals(m, p, nb, q, q2, mx, red)) return;
        if (tid == 0) {
            MinState &o = st[p];
            const double step = s.step / mz.scale;
            o.step = step;
            o.evals = s.evals + 1;
            if (!(mx >= mz.xtol / step)) o.success = s.success | 1;
        }
    }
}

__global__ void k_count_active(const MinState *st, int npairs, int *count)
{
    int c = 0;
    for (int p = threadIdx.x; p < npairs; p += blockDim.x) c += st[p].done ? 0 : 1;
    c = __reduce_add_sync(0xffffffffu, c);
    if (threadIdx.x == 0) *count = c;
}

struct PairRun {
    mgr_level_desc full{};
    int size[3] = {1, 1, 1}, prev[3] = {0, 0, 0}, csize[3] = {1, 1, 1};
    DevBuf<float> src, ref, src_n, ref_n;
    std::vector<double> params;
    mgr_level *lvl = nullptr;
    mgr_level *lvl0 = nullptr;       // the pass-0 level while lvl (refine pass) uses its images
    std::vector<mgr_level *> made;   // per level (index shift): made ahead, not yet in use
    std::vector<mgr_level *> made1;  // per level: the refine pass's level on made[shift]'s images
    bool x_on_device = false;        // x holds the parameters of the next pass (params only sized)
    DevBuf<double> x, g, xt, gt, costs;
    bool identity = false;   // both images of one value
    bool in_pass = false;
    double cost = 0.0;
    int evals = 0;
    ~PairRun()
    {
        if (lvl) mgr_level_destroy(lvl);
        if (lvl0) mgr_level_destroy(lvl0);
        for (mgr_level *m : made1)
            if (m) mgr_level_destroy(m);
        for (mgr_level *m : made)
            if (m) mgr_level_destroy(m);
    }
};

// run f(i) for i < n on host threads (the per-pair coefficient resampling
// is independent host work); the first exception is rethrown
template <class F>
void parallel_pairs(size_t n, F f)
{
    const size_t nt = std::max<size_t>(1, std::min<size_t>(n, std::thread::hardware_concurrency()));
    std::vector<std::exception_ptr> err(nt);
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            try {
                for (size_t i = t; i < n; i += nt) f(i);
            } catch (...) {
                err[t] = std::current_exception();
            }
        });
    for (auto &x : th) x.join();
    for (auto &e : err)
        if (e) std::rethrow_exception(e);
}

void ckm(mgr_status s)
{
    if (s == MGR_ERR_ARG) throw std::invalid_argument(mgr_last_error());
    if (s == MGR_ERR_TIMEOUT) throw TimeoutError(mgr_last_error());
    if (s == MGR_ERR_OOM) throw std::bad_alloc();
    if (s != MGR_OK) throw std::runtime_error(mgr_last_error());
}

// Run the minimizer of every pair with in_pass set, in lock step, until all
// have finished.  Steps are captured into a CUDA graph when use_graphs.
void run_pass(std::vector<std::unique_ptr<PairRun>> &pairs, const mgr_minimizer_desc &mz, int dim, int tile[3],
              bool use_graphs, bool persistent, cudaStream_t st, const char *label)
{
    std::vector<int> members;
    for (size_t i = 0; i < pairs.size(); ++i)
        if (pairs[i]->in_pass) members.push_back(int(i));
    const int np = int(members.size());
    if (np == 0) return;
    TraceScope tr_setup("batch: pass setup", st);
    std::vector<EvalArgs> args(np);
    std::vector<PairVec> vecs(np);
    std::vector<MinState> states(np);
    std::vector<int2> titems, gitems;
    std::vector<int> nblocks(np);
    size_t sm_warp = 0, sm_adj = 0, max_params = 0;
    int has_pen = 0;
    for (int k = 0; k < np; ++k) {
        PairRun &r = *pairs[members[k]];
        const size_t n = r.params.size();
        if (r.x_on_device) r.x.alloc(n, st);   // (already there: the refine wrote it)
        else r.x.upload(r.params, st);
        r.x_on_device = false;
        r.g.alloc(n, st);
        r.xt.alloc(n, st);
        r.gt.alloc(n, st);
        r.costs.alloc(2, st);
        EvalArgs a = r.lvl->args();
        a.params = r.xt.p;
        a.grad_total = r.gt.p;
        a.grad_image = nullptr;
        a.grad_penalty = nullptr;
        a.costs = r.costs.p;
        args[k] = a;
        vecs[k] = PairVec{r.x.p, r.g.p, r.xt.p, r.gt.p, r.costs.p, int(n), dim == 3 ? a.params_f : nullptr};
        MinState s{};
        s.step = mz.step;
        states[k] = s;
        const int nt = a.ax[0].nt * a.ax[1].nt * (dim == 3 ? a.ax[2].nt : 1);
        for (int t = 0; t < nt; ++t) titems.push_back(make_int2(k, t));
        nblocks[k] = gather_blocks(a);
        for (int b = 0; b < nblocks[k]; ++b) gitems.push_back(make_int2(k, b));
        sm_warp = std::max(sm_warp, split_smem(a, 0));
        sm_adj = std::max(sm_adj, split_smem(a, 1));
        has_pen |= a.has_penalty;
        max_params = std::max(max_params, n);
    }
    if (std::max(sm_warp, sm_adj) > 200 * 1024)
        throw std::invalid_argument("coefficient spacing too small for the batched tile shape");
    // the pass's tables and counters in one device buffer, filled by one
    // upload (the counters and flags are zero)
    MinScratch msc;
    msc.nblk = int((max_params + MCH - 1) / MCH);
    size_t bytes = 0;
    auto place = [&](size_t sz) {
        const size_t o = bytes;
        bytes = (bytes + sz + 255) & ~size_t(255);
        return o;
    };
    const size_t o_args = place(sizeof(EvalArgs) * np), o_vecs = place(sizeof(PairVec) * np);
    const size_t o_states = place(sizeof(MinState) * np), o_titems = place(sizeof(int2) * titems.size());
    const size_t o_gitems = place(sizeof(int2) * gitems.size()), o_nblocks = place(sizeof(int) * np);
    const size_t o_active = place(sizeof(int) * np), o_count = place(sizeof(int));
    const size_t o_moved = place(sizeof(int) * np), o_mcount = place(sizeof(unsigned) * np);
    const size_t o_queue = place(sizeof(int) * 4);   // the persistent kernels' queues (warp, adjoint)
    const size_t o_mpart = place(sizeof(double) * size_t(np) * msc.nblk * 3);
    std::vector<unsigned char> blob(o_mpart, 0);
    std::memcpy(blob.data() + o_args, args.data(), sizeof(EvalArgs) * np);
    std::memcpy(blob.data() + o_vecs, vecs.data(), sizeof(PairVec) * np);
    std::memcpy(blob.data() + o_states, states.data(), sizeof(MinState) * np);
    std::memcpy(blob.data() + o_titems, titems.data(), sizeof(int2) * titems.size());
    std::memcpy(blob.data() + o_gitems, gitems.data(), sizeof(int2) * gitems.size());
    std::memcpy(blob.data() + o_nblocks, nblocks.data(), sizeof(int) * np);
    DevBuf<unsigned char> d_pass;
    d_pass.alloc(bytes, st);
    ck(cudaMemcpyAsync(d_pass.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, st), "pass tables H2D");
    EvalArgs *d_args = reinterpret_cast<EvalArgs *>(d_pass.p + o_args);
    PairVec *d_vecs = reinterpret_cast<PairVec *>(d_pass.p + o_vecs);
    MinState *d_states = reinterpret_cast<MinState *>(d_pass.p + o_states);
    int2 *d_titems = reinterpret_cast<int2 *>(d_pass.p + o_titems);
    int2 *d_gitems = reinterpret_cast<int2 *>(d_pass.p + o_gitems);
    int *d_nblocks = reinterpret_cast<int *>(d_pass.p + o_nblocks);
    int *d_active = reinterpret_cast<int *>(d_pass.p + o_active);
    int *d_count = reinterpret_cast<int *>(d_pass.p + o_count);
    int *d_queue = reinterpret_cast<int *>(d_pass.p + o_queue);
    msc.part = reinterpret_cast<double *>(d_pass.p + o_mpart);
    msc.count = reinterpret_cast<unsigned *>(d_pass.p + o_mcount);
    msc.moved = reinterpret_cast<int *>(d_pass.p + o_moved);
    const dim3 mgrid(msc.nblk, np);

    // persistent launches (3D): as many blocks as stay resident, drawing
    // (pair, tile) items from the device queue; the grid sizes are fixed
    // before any capture
    const bool queue = persistent && dim == 3;
    int qgrid[2] = {0, 0};
    if (queue) {
        prepare_split_batch(dim, tile[0], tile[1], tile[2], sm_warp, sm_adj);
        qgrid[0] = std::min(int(titems.size()), split3_queue_grid(tile[2], 0, sm_warp));
        qgrid[1] = std::min(int(titems.size()), split3_queue_grid(tile[2], 1, sm_adj));
    }
    auto step = [&]() {
        k_min_propose<<<mgrid, MT, 0, st>>>(d_states, d_vecs, mz, d_active, msc);
        if (queue) {
            launch_split3_queue(tile[2], d_args, d_titems, int(titems.size()), d_active, d_queue, qgrid[0], sm_warp,
                                0, st);
            launch_split3_queue(tile[2], d_args, d_titems, int(titems.size()), d_active, d_queue + 2, qgrid[1], sm_adj,
                                1, st);
        } else {
            if (!launch_split_batch(dim, tile[0], tile[1], tile[2], d_args, d_titems, int(titems.size()),
                                    d_active, sm_warp, 0, st))
                throw std::invalid_argument("tile shape not compiled in");
            launch_split_batch(dim, tile[0], tile[1], tile[2], d_args, d_titems, int(titems.size()),
                               d_active, sm_adj, 1, st);
        }
        launch_gather_batch(dim, d_args, d_gitems, int(gitems.size()), d_active, d_nblocks, has_pen, st);
        k_min_update<<<mgrid, MT, 0, st>>>(d_states, d_vecs, mz, d_active, msc);
        count_launch(2);
    };
    const int chunk = 8;
    const int max_steps = 1 + (mz.maxiter + 2) * 64;   // bounded: GSL trials shrink the step geometrically
    // kernel attributes are set outside the capture
    prepare_split_batch(dim, tile[0], tile[1], tile[2], sm_warp, sm_adj);
    cudaGraphExec_t exec = nullptr;
    const unsigned kernels_per_chunk = unsigned(chunk) * 5 + 1;
    tr_setup.stop();
    if (use_graphs) {
        TraceScope tr("batch: graph capture", st);
        cudaGraph_t graph = nullptr;
        ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "capture");
        // launches recorded during capture run only when the graph runs
        count_launch_pause(true);
        try {
            for (int i = 0; i < chunk; ++i) step();
        } catch (...) {
            count_launch_pause(false);
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        k_count_active<<<1, 32, 0, st>>>(d_states, np, d_count);
        count_launch_pause(false);
        ck(cudaStreamEndCapture(st, &graph), "end capture");
        ck(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
        cudaGraphDestroy(graph);
    }
    TraceScope tr_steps("batch: steps", st);
    int steps = 0;
    while (steps < max_steps) {
        if (use_graphs) {
            ck(cudaGraphLaunch(exec, st), "graph launch");
            count_launch(kernels_per_chunk);
        } else {
            for (int i = 0; i < chunk; ++i) step();
            k_count_active<<<1, 32, 0, st>>>(d_states, np, d_count);
            count_launch();
        }
        steps += chunk;
        int active = 0;
        ck(cudaMemcpyAsync(&active, d_count, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "batch sync");
        if (active == 0) break;
    }
    const auto t_steps0 = tr_steps.t0;
    tr_steps.stop();
    const double steps_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_steps0).count();
    TraceScope tr_back("batch: readback", st);
    if (exec) cudaGraphExecDestroy(exec);
    ck(cudaMemcpyAsync(states.data(), d_states, np * sizeof(MinState), cudaMemcpyDeviceToHost, st), "D2H");
    // every pair's parameters and status flag (counters[6] of its level)
    // gathered on the device, so that one copy brings them back
    std::vector<size_t> off(np + 1, 0);
    for (int k = 0; k < np; ++k) off[k + 1] = off[k] + pairs[members[k]]->params.size();
    const size_t flags_at = off[np] * sizeof(double);
    DevBuf<unsigned char> d_back;
    d_back.alloc(flags_at + size_t(np) * sizeof(unsigned), st);
    for (int k = 0; k < np; ++k) {
        PairRun &r = *pairs[members[k]];
        ck(cudaMemcpyAsync(d_back.p + off[k] * sizeof(double), r.x.p, r.params.size() * sizeof(double),
                           cudaMemcpyDeviceToDevice, st),
           "gather");
        ck(cudaMemcpyAsync(d_back.p + flags_at + size_t(k) * sizeof(unsigned), r.lvl->counters.p + 6,
                           sizeof(unsigned), cudaMemcpyDeviceToDevice, st),
           "gather");
    }
    std::vector<unsigned char> back(d_back.n);
    ck(cudaMemcpyAsync(back.data(), d_back.p, back.size(), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "batch sync");
    std::vector<unsigned> flags(np, 0u);
    for (int k = 0; k < np; ++k) {
        PairRun &r = *pairs[members[k]];
        std::memcpy(r.params.data(), back.data() + off[k] * sizeof(double), r.params.size() * sizeof(double));
        std::memcpy(&flags[k], back.data() + flags_at + size_t(k) * sizeof(unsigned), sizeof(unsigned));
    }
    for (int k = 0; k < np; ++k) throw_if_flagged(pairs[members[k]]->lvl, flags[k]);
    double vox_evals = 0.0;
    for (int k = 0; k < np; ++k) {
        PairRun &r = *pairs[members[k]];
        r.cost = states[k].f;
        r.evals += states[k].evals;
        vox_evals += double(states[k].evals) * double(args[k].n[0]) * args[k].n[1] * args[k].n[2];
        round_params_to_float(r.params);
    }
    tr_back.stop();
    if (trace_enabled()) {
        const std::string tag = "batch: " + std::string(label) + " ";
        trace_count((tag + "Mvoxel-evals").c_str(), vox_evals * 1e-6);
        trace_count((tag + "lock-step steps").c_str(), double(steps));
        trace_count((tag + "steps ms").c_str(), steps_ms);
    }
}

}  // namespace

}  // namespace mgr

using namespace mgr;

namespace {

// images_on_device: srcs/refs are device pointers of this device
mgr_status register_batch(int npairs, const mgr_level_desc *descs, int levels, const mgr_minimizer_desc *mz,
                          const float *const *srcs, const float *const *refs, bool images_on_device, int device,
                          int use_graphs, double *const *params_out, const size_t *max_params, int *csize_out,
                          double *final_costs, int *evaluations)
{
    if (npairs < 1 || !descs || !mz || !srcs || !refs || !params_out || !max_params || !csize_out) {
        set_last_error("mgr_register_batch: invalid argument");
        return MGR_ERR_ARG;
    }
    try {
        if (levels < 1) throw std::invalid_argument("levels must be >= 1");
        const int dim = descs[0].dim;
        if (dim != 2 && dim != 3) throw std::invalid_argument("dim must be 2 or 3");
        if (mz->maxiter < 1) throw std::invalid_argument("maxiter must be >= 1");
        for (int p = 0; p < npairs; ++p) {
            if (!srcs[p] || !refs[p] || !params_out[p]) throw std::invalid_argument("null image or output pointer");
            const mgr_level_desc &d = descs[p];
            if (d.dim != dim) throw std::invalid_argument("all pairs of a batch must have the same dimension");
            if (d.cost != descs[0].cost || d.has_penalty != descs[0].has_penalty)
                throw std::invalid_argument("all pairs of a batch must use the same cost and penalty");
            for (int k = 0; k < dim; ++k) {
                if (d.csize[k] != 0) throw std::invalid_argument("the batch derives the grids from the rate");
                if (d.size[k] < 2) throw std::invalid_argument("image dimensions must be >= 2");
            }
        }
        if (mz->kind != MGR_MIN_GSL_SD && mz->kind != MGR_MIN_GDSQ) throw std::invalid_argument("unknown minimizer");
        ck(cudaSetDevice(device), "cudaSetDevice");
        configure_pool(device);
        cudaStream_t st;
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } guard{st};
        // the workers that make the levels ahead, each on its own stream (the
        // streams outlive the pairs: levels not yet moved to st free their
        // buffers on them); four: eight measured no faster for the 3D cohort
        // and slower for the 60-frame series (their CUDA calls contend with
        // the main thread's)
        const int nworkers = int(std::max<size_t>(
            1, std::min<size_t>({size_t(4), size_t(npairs), size_t(std::max(1u, std::thread::hardware_concurrency()))})));
        struct StreamsGuard {
            std::vector<cudaStream_t> s;
            ~StreamsGuard()
            {
                for (cudaStream_t x : s) cudaStreamDestroy(x);
            }
        } st_prep;
        for (int w = 0; w < nworkers; ++w) {
            cudaStream_t x;
            ck(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), "cudaStreamCreate");
            st_prep.s.push_back(x);
        }
        // events.e[w * levels + shift]: worker w made level `shift`;
        // events.e[nworkers * levels]: the normalised images are on st
        struct EventGuard {
            std::vector<cudaEvent_t> e;
            ~EventGuard()
            {
                for (cudaEvent_t x : e) cudaEventDestroy(x);
            }
        } events;
        // events.e[ev_retired + shift]: st is done with the levels retired
        // when level `shift` starts
        events.e.assign(size_t(nworkers) * levels + 1 + levels, nullptr);
        for (auto &e : events.e) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        const size_t ev_normalized = size_t(nworkers) * levels;
        const size_t ev_retired = ev_normalized + 1;
        // one tile for all pairs and levels (the batch kernels take one
        // shape): the registration drivers' tile
        std::array<int, 3> rt;
        registration_tile(dim, rt.data());
        std::vector<std::array<int, 3>> level_tile(levels, rt);
        // levels the pairs have left are destroyed on a helper thread while
        // the next passes run.  Their buffers are freed on a stream other
        // than st, ordered after their last use by an event on st: st may be
        // capturing a graph meanwhile, and a capture takes in work that any
        // thread queues on the stream.
        struct Reaper {
            std::vector<mgr_level *> pending;
            std::thread t;
            void join()
            {
                if (t.joinable()) t.join();
            }
            void launch()
            {
                join();
                std::vector<mgr_level *> v;
                v.swap(pending);
                if (!v.empty())
                    t = std::thread([v] {
                        for (mgr_level *L : v) mgr_level_destroy(L);
                    });
            }
            ~Reaper()
            {
                join();
                for (mgr_level *L : pending) mgr_level_destroy(L);
            }
        } reaper;
        std::vector<std::unique_ptr<PairRun>> pairs;
        TraceScope tr_in("batch: input+normalize", st);
        std::vector<const float *> in_src(npairs), in_ref(npairs);
        std::vector<float *> out_src(npairs), out_ref(npairs);
        std::vector<size_t> nvox(npairs);
        // host images on a device that reads pageable host memory
        // coherently (address translation through the host's page tables,
        // as on Grace-based systems): the normalisation kernels read the
        // caller's arrays where they are, with no staged copy (one read of
        // the images over the CPU-GPU link);
        // MGR_HOST_COPY=1 keeps the copies
        const bool direct = !images_on_device && coherent_host_access(device);
        trace_count("batch: images read in place (1 = yes)", direct ? 1.0 : 0.0);
        for (int p = 0; p < npairs; ++p) {
            std::unique_ptr<PairRun> r(new PairRun);
            r->full = descs[p];
            const size_t n = size_t(descs[p].size[0]) * descs[p].size[1] * (dim == 3 ? descs[p].size[2] : 1);
            r->src_n.alloc(n, st);
            r->ref_n.alloc(n, st);
            in_src[p] = srcs[p];
            in_ref[p] = refs[p];
            if (!images_on_device && !direct) {
                r->src.alloc(n, st);
                r->ref.alloc(n, st);
                in_src[p] = r->src.p;
                in_ref[p] = r->ref.p;
            }
            out_src[p] = r->src_n.p;
            out_ref[p] = r->ref_n.p;
            nvox[p] = n;
            pairs.push_back(std::move(r));
        }
        if (!images_on_device && !direct) {
            // host images: the copies from pageable memory are staged by the
            // calling thread, so the pairs are uploaded from several host
            // threads, each on its own per-thread stream
            ck(cudaStreamSynchronize(st), "sync");   // (the buffers were allocated in st's order)
            parallel_pairs(size_t(npairs), [&](size_t p) {
                ck(cudaSetDevice(device), "cudaSetDevice");
                const size_t bytes = nvox[p] * sizeof(float);
                ck(cudaMemcpyAsync(pairs[p]->src.p, srcs[p], bytes, cudaMemcpyHostToDevice, cudaStreamPerThread),
                   "H2D");
                ck(cudaMemcpyAsync(pairs[p]->ref.p, refs[p], bytes, cudaMemcpyHostToDevice, cudaStreamPerThread),
                   "H2D");
                ck(cudaStreamSynchronize(cudaStreamPerThread), "H2D sync");
            });
        }
        // images read in place: the sums pass also copies them to the
        // device, so that they cross the CPU-GPU link once
        const std::vector<char> varied = normalize_pairs(in_src, in_ref, nvox, out_src, out_ref, st, direct);
        for (int p = 0; p < npairs; ++p) {
            PairRun &r = *pairs[p];
            r.src.release();   // the uploaded images are no longer read (stream-ordered free)
            r.ref.release();
            r.identity = !varied[p];
            if (r.identity) {
                for (int k = 0; k < 3; ++k)
                    r.csize[k] = k < dim ? csize_from_rate(descs[p].size[k], descs[p].rate[k]) : 1;
                r.params.assign(size_t(r.csize[0]) * r.csize[1] * r.csize[2] * dim, 0.0);
            }
        }
        tr_in.stop();
        for (auto &rp : pairs) {
            rp->made.assign(levels, nullptr);
            rp->made1.assign(levels, nullptr);
        }
        // The images and the first level object of every level depend only
        // on the normalised images, not on the parameters: worker threads
        // make them (worker w the pairs i = w mod nworkers, on its own
        // stream), coarsest level first, while the minimizers of the coarser
        // levels run on st.  A level is ready once every worker has made it:
        // made[shift] counts them on the host, the workers' events mark it
        // on the device.
        ck(cudaEventRecord(events.e[ev_normalized], st), "cudaEventRecord");
        struct Prep {
            std::mutex mu;
            std::condition_variable cv;
            std::vector<int> made;
            std::exception_ptr err;
            std::atomic<bool> stop{false};
        } prep;
        prep.made.assign(levels, 0);
        struct Joiner {   // before the pairs go: the workers end and their device work drains
            Prep &p;
            std::vector<cudaStream_t> s;
            std::vector<std::thread> t;
            ~Joiner()
            {
                p.stop = true;
                for (auto &x : t)
                    if (x.joinable()) x.join();
                for (cudaStream_t x : s) cudaStreamSynchronize(x);
            }
        } workers{prep, st_prep.s, {}};
        auto make_levels = [&](int w) {
            cudaStream_t sp = st_prep.s[w];
            try {
                ck(cudaSetDevice(device), "cudaSetDevice");
                ck(cudaStreamWaitEvent(sp, events.e[ev_normalized], 0), "cudaStreamWaitEvent");
                // the grid each level starts with: the coarsest level's from
                // the rate, then the grid the previous level ended with (its
                // refine pass grows it or keeps it; upscaling keeps it)
                std::vector<std::array<int, 3>> grid(pairs.size(), std::array<int, 3>{1, 1, 1});
                for (int shift = levels - 1; shift >= 0 && !prep.stop; --shift) {
                    TraceScope tr_make("batch: levels made ahead (workers)", sp);
                    for (size_t i = size_t(w); i < pairs.size(); i += size_t(nworkers)) {
                        PairRun &r = *pairs[i];
                        if (r.identity) continue;
                        int size[3] = {1, 1, 1}, ncn[3] = {1, 1, 1};
                        int *csize = grid[i].data();
                        for (int k = 0; k < dim; ++k) {
                            size[k] = r.full.size[k] / (1 << shift);
                            if (shift == levels - 1) {
                                csize[k] = csize_from_rate(size[k], r.full.rate[k]);
                                if (csize[k] - 2 <= 1)
                                    throw std::invalid_argument("coefficient rate too large for the coarsest level");
                            }
                            ncn[k] = refine_csize(size[k], r.full.rate[k]);
                        }
                        const size_t n = size_t(size[0]) * size[1] * (dim == 3 ? size[2] : 1);
                        DevBuf<float> src_l, ref_l;   // freed in stream order after the level's copies
                        src_l.alloc(n, sp);
                        ref_l.alloc(n, sp);
                        scale_image(r.src_n.p, r.full.size, src_l.p, size, dim, sp);
                        scale_image(r.ref_n.p, r.full.size, ref_l.p, size, dim, sp);
                        mgr_level_desc d = r.full;
                        for (int k = 0; k < 3; ++k) {
                            d.size[k] = k < dim ? size[k] : 1;
                            d.csize[k] = k < dim ? csize[k] : 0;
                        }
                        mgr_level *L = nullptr;
                        ckm(mgr_level_create(&d, device, sp, &L));
                        r.made[shift] = L;
                        const int *tile = level_tile[shift].data();
                        ckm(mgr_level_set_path(L, MGR_PATH_SPLIT, tile[0], tile[1], tile[2]));
                        level_set_images_async(L, src_l.p, ref_l.p);
                        if (refine_grows(dim, csize, ncn)) {
                            // the refine pass's grid, on the same images
                            r.made1[shift] = level_create_on_images(L, ncn, sp);
                            for (int k = 0; k < dim; ++k) csize[k] = ncn[k];
                        }
                    }
                    ck(cudaEventRecord(events.e[size_t(w) * levels + shift], sp), "cudaEventRecord");
                    tr_make.stop();
                    std::lock_guard<std::mutex> lk(prep.mu);
                    prep.made[shift] += 1;
                    prep.cv.notify_all();
                }
            } catch (...) {
                std::lock_guard<std::mutex> lk(prep.mu);
                if (!prep.err) prep.err = std::current_exception();
                prep.cv.notify_all();
            }
        };
        for (int w = 0; w < nworkers; ++w) workers.t.emplace_back(make_levels, w);
        for (int shift = levels - 1; shift >= 0; --shift) {
            TraceScope tr_scale("batch: upscale", st);
            for (auto &rp : pairs) {   // (a scaling of the coefficients: cheaper than threads)
                PairRun &r = *rp;
                r.in_pass = false;
                if (r.identity) continue;
                for (int k = 0; k < dim; ++k) r.size[k] = r.full.size[k] / (1 << shift);
                if (shift == levels - 1) {
                    for (int k = 0; k < 3; ++k) r.csize[k] = k < dim ? csize_from_rate(r.size[k], r.full.rate[k]) : 1;
                    r.params.assign(size_t(r.csize[0]) * r.csize[1] * r.csize[2] * dim, 0.0);
                } else {
                    upscale_params(dim, r.prev, r.size, r.params);
                }
            }
            tr_scale.stop();
            {
                TraceScope tr_wait("batch: wait for the level", st);
                std::unique_lock<std::mutex> lk(prep.mu);
                prep.cv.wait(lk, [&] { return prep.err || prep.made[shift] == nworkers; });
                if (prep.err) std::rethrow_exception(prep.err);
                lk.unlock();
                for (int w = 0; w < nworkers; ++w)
                    ck(cudaStreamWaitEvent(st, events.e[size_t(w) * levels + shift], 0), "cudaStreamWaitEvent");
            }
            int *tile = level_tile[shift].data();
            for (int pass = 0; pass < 2; ++pass) {
                TraceScope tr_lvl("batch: refine+level setup", st);
                if (pass == 1) {
                    // refine: whether a pair's grid grows follows from the
                    // sizes; the coefficients of the pass-0 result (r.x) are
                    // refined on the device for all growing pairs at once and
                    // stay there for the next pass (the host copy is only
                    // resized: the pass's readback refreshes it).  Grids
                    // with an axis of fewer than 4 coefficients are refined
                    // on the host.
                    std::vector<RefineJobSpec> jobs;
                    std::vector<PairRun *> on_dev;
                    std::vector<size_t> at;
                    size_t total = 0;
                    for (auto &rp : pairs) {
                        PairRun &r = *rp;
                        if (r.identity) continue;
                        int ncn[3] = {1, 1, 1};
                        for (int k = 0; k < dim; ++k) ncn[k] = refine_csize(r.size[k], r.full.rate[k]);
                        r.in_pass = refine_grows(dim, r.csize, ncn);
                        if (!r.in_pass) continue;
                        bool small = false;
                        for (int k = 0; k < dim; ++k) small |= r.csize[k] < 4 || ncn[k] < 4;
                        if (small) {
                            refine_params(dim, r.csize, ncn, r.params);
                        } else {
                            RefineJobSpec j;
                            for (int k = 0; k < 3; ++k) {
                                j.nc_old[k] = r.csize[k];
                                j.nc_new[k] = ncn[k];
                            }
                            j.in = r.x.p;
                            j.out = nullptr;
                            jobs.push_back(j);
                            on_dev.push_back(&r);
                            at.push_back(total);
                            total += size_t(ncn[0]) * ncn[1] * ncn[2] * dim;
                        }
                        for (int k = 0; k < 3; ++k) r.csize[k] = ncn[k];
                    }
                    if (!jobs.empty()) {
                        DevBuf<double> d_new;
                        d_new.alloc(total, st);
                        for (size_t j = 0; j < jobs.size(); ++j) jobs[j].out = d_new.p + at[j];
                        refine_params_device(dim, jobs, st);
                        for (size_t j = 0; j < jobs.size(); ++j) {
                            PairRun &r = *on_dev[j];
                            const size_t n = size_t(r.csize[0]) * r.csize[1] * r.csize[2] * dim;
                            r.x.alloc(n, st);   // (the old buffer is freed after the refine read it)
                            ck(cudaMemcpyAsync(r.x.p, d_new.p + at[j], n * sizeof(double), cudaMemcpyDeviceToDevice,
                                               st),
                               "refined parameters");
                            r.params.resize(n);
                            r.x_on_device = true;
                        }
                    }
                }
                TraceScope tr_grid(pass == 1 ? "batch: set grid (refine pass)" : "batch: destroy+take level", st);
                for (auto &rp : pairs) {
                    PairRun &r = *rp;
                    if (r.identity) continue;
                    if (pass == 1) {
                        // same images as pass 0, the refined grid: the level
                        // made ahead on pass 0's images, else a new grid on
                        // the pass-0 level
                        if (!r.in_pass) continue;
                        mgr_level *L1 = r.made1[shift];
                        if (L1 && L1->nc[0] == r.csize[0] && L1->nc[1] == r.csize[1] &&
                            (dim == 2 || L1->nc[2] == r.csize[2])) {
                            r.made1[shift] = nullptr;
                            r.lvl0 = r.lvl;
                            r.lvl = L1;
                            L1->rebind(st);
                        } else {
                            level_set_grid(r.lvl, r.csize, tile);
                        }
                        continue;
                    }
                    r.in_pass = true;
                    if (r.lvl) reaper.pending.push_back(r.lvl);
                    if (r.lvl0) reaper.pending.push_back(r.lvl0);
                    r.lvl0 = nullptr;
                    r.lvl = r.made[shift];
                    r.made[shift] = nullptr;
                    r.lvl->rebind(st);
                    // the level was made with the grid of this size; the
                    // parameters carried over from the coarser level keep theirs
                    if (r.lvl->nc[0] != r.csize[0] || r.lvl->nc[1] != r.csize[1] ||
                        (dim == 3 && r.lvl->nc[2] != r.csize[2]))
                        level_set_grid(r.lvl, r.csize, tile);
                }
                if (pass == 0 && !reaper.pending.empty()) {
                    cudaStream_t sr = st_prep.s[0];
                    ck(cudaEventRecord(events.e[ev_retired + shift], st), "cudaEventRecord");
                    ck(cudaStreamWaitEvent(sr, events.e[ev_retired + shift], 0), "cudaStreamWaitEvent");
                    for (mgr_level *L : reaper.pending) L->rebind(sr);
                    reaper.launch();
                }
                tr_grid.stop();
                tr_lvl.stop();
                const std::string label = "level " + std::to_string(shift) + " pass " + std::to_string(pass);
                run_pass(pairs, *mz, dim, tile, (use_graphs & 1) != 0, (use_graphs & 2) != 0, st, label.c_str());
            }
            for (auto &rp : pairs)
                for (int k = 0; k < 3; ++k) rp->prev[k] = rp->size[k];
        }
        trace_report("mgr_register_batch");
        for (int p = 0; p < npairs; ++p) {
            PairRun &r = *pairs[p];
            if (r.params.size() > max_params[p]) throw std::invalid_argument("params_out too small");
            std::copy(r.params.begin(), r.params.end(), params_out[p]);
            for (int k = 0; k < 3; ++k) csize_out[p * 3 + k] = r.csize[k];
            if (final_costs) final_costs[p] = r.cost;
            if (evaluations) evaluations[p] = r.evals;
        }
        return MGR_OK;
    } catch (const std::invalid_argument &e) {
        set_last_error(e.what());
        return MGR_ERR_ARG;
    } catch (const TimeoutError &e) {
        set_last_error(e.what());
        return MGR_ERR_TIMEOUT;
    } catch (const std::bad_alloc &) {
        set_last_error("allocation failed");
        return MGR_ERR_OOM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MGR_ERR_CUDA;
    }
}

}  // namespace

extern "C" mgr_status mgr_register_batch(int npairs, const mgr_level_desc *descs, int levels,
                                         const mgr_minimizer_desc *mz, const float *const *srcs,
                                         const float *const *refs, int device, int use_graphs,
                                         double *const *params_out, const size_t *max_params, int *csize_out,
                                         double *final_costs, int *evaluations)
{
    return register_batch(npairs, descs, levels, mz, srcs, refs, false, device, use_graphs, params_out, max_params,
                          csize_out, final_costs, evaluations);
}

extern "C" mgr_status mgr_register_batch_device(int npairs, const mgr_level_desc *descs, int levels,
                                                const mgr_minimizer_desc *mz, const float *const *d_srcs,
                                                const float *const *d_refs, int device, int use_graphs,
                                                double *const *params_out, const size_t *max_params,
                                                int *csize_out, double *final_costs, int *evaluations)
{
    return register_batch(npairs, descs, levels, mz, d_srcs, d_refs, true, device, use_graphs, params_out,
                          max_params, csize_out, final_costs, evaluations);
}
