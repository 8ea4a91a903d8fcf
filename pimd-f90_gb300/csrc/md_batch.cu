// md_batch.cu -- many independent ring polymers (replicas) of uneven sizes stepped together.
//
// The reference runs one ring polymer per MPI job (PIMD.f90; MD.f90:35-110 per step). Here a
// batch holds any number of replicas, each with its own molecule count, bead count and
// temperature. Replicas that share a box (same molecule count, box and cutoff) are stacked on
// the bead axis of one force-engine context, so every force kernel covers all beads of all
// those replicas in one launch; the normal-mode, thermostat and kick work of all replicas (own P,
// own NM matrices and Langevin coefficients at its own temperature) runs in one launch per phase
// of the step, each block on one replica's atoms. A step of the whole batch is one CUDA graph:
// the integrator up to the force call, one branch per box group on its own stream (each with its
// dipole loop as a conditional while node), then the integrator after it and the step outputs.
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "engine.h"

namespace pimd {
int run_forces(Engine &E, int t, int check_every, double *Upott, double *virialt, double *virialct, double *virt9);
__global__ void k_set_step(int *dstep, int t);
}  // namespace pimd

using namespace pimd;

namespace {

struct BatchReplica {
    int group, local, bead0, P, natoms;
    double temp, box0;
    double *d_C = nullptr, *d_A = nullptr;
    unsigned long long seed;
};

struct BatchGroup {
    pimd_ctx *ctx = nullptr;
    std::vector<int> reps;
    int Ptot = 0, natoms = 0;
    double *RRt = nullptr, *PPt = nullptr, *dRRt = nullptr, *RRc = nullptr;
};

}  // namespace

struct pimd_batch {
    std::vector<BatchGroup> groups;
    std::vector<BatchReplica> reps;
    pimd_md_params mp{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev_join;
    cudaGraphExec_t gexec = nullptr;
    double *d_out4 = nullptr, *d_uk = nullptr;
    // the integrator of every replica in one launch per phase: per-replica arguments, the block map
    // (replica, block of its own grid) and the step-output table
    NMBatchRep *d_reps = nullptr;
    int2 *d_blkmap = nullptr;
    NMSumRep *d_sums = nullptr;
    int nblk = 0;
    size_t smem = 0;
    bool fast = false;
    std::vector<void *> allocs;
    int t = 0;
    std::string err;
};

static int bfail(pimd_batch *bt, int code, const std::string &msg) {
    bt->err = msg;
    return code;
}

static int bcuda(pimd_batch *bt, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PIMD_OK;
    return bfail(bt, e == cudaErrorMemoryAllocation ? PIMD_ERR_NOMEM : PIMD_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
static int balloc(pimd_batch *bt, T **p, size_t n) {
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return bcuda(bt, e, "cudaMalloc");
    bt->allocs.push_back(*p);
    cudaMemset(*p, 0, sizeof(T) * (n ? n : 1));
    return PIMD_OK;
}

static NMArgs replica_args(const pimd_batch *bt, const BatchReplica &r, const Engine &E) {
    NMArgs a{};
    a.P = r.P;
    a.natoms = r.natoms;
    a.C = r.d_C;
    a.A = r.d_A;
    a.massO = bt->mp.massO;
    a.massH = bt->mp.massH;
    a.delt = bt->mp.delt;
    a.delt2 = bt->mp.delt / 2.0;
    a.box0 = r.box0;
    a.boxi0 = 1.0 / r.box0;
    a.langevin = bt->mp.langevin;
    a.evolve = r.P > 1;
    a.seed = r.seed;
    a.tstep = E.kp.dstep;
    a.fast = E.precision == PIMD_MIXED;
    return a;
}

// One PIMD_VV step of every replica (MD.f90:35-110): the integrator of all replicas up to the
// force call in one launch, the force call of each box group on the group context's stream (one
// graph branch per group, each with its dipole loop as a conditional node), then the integrator
// after it and the step outputs of all replicas, one launch each.
static int capture_batch(pimd_batch *bt) {
    cudaError_t e = cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bcuda(bt, e, "batch capture");
    cudaMemsetAsync(bt->d_uk, 0, sizeof(double) * bt->reps.size(), bt->stream);
    nm_launch_md_batch(0, bt->fast, bt->nblk, bt->smem, bt->stream, bt->d_reps, bt->d_blkmap);
    cudaEventRecord(bt->ev_fork, bt->stream);
    int rc = PIMD_OK;
    for (size_t gi = 0; gi < bt->groups.size() && !rc; gi++) {
        BatchGroup &g = bt->groups[gi];
        Engine &E = g.ctx->E;
        cudaStreamWaitEvent(E.stream, bt->ev_fork, 0);
        if (!E.body_stream) cudaStreamCreateWithFlags(&E.body_stream, cudaStreamNonBlocking);
        const bool timers_on = E.timers.on;
        E.timers.on = false;
        E.capturing = true;
        double *d = E.d_out;  // Upott, virialt, virialct of all beads of the group
        rc = run_forces(E, 0, 0, d, d + g.Ptot, d + 2 * g.Ptot, nullptr);
        if (rc) bt->err = E.last_error;
        E.capturing = false;
        E.timers.on = timers_on;
        cudaEventRecord(bt->ev_join[gi], E.stream);
        cudaStreamWaitEvent(bt->stream, bt->ev_join[gi], 0);
    }
    nm_launch_md_batch(1, bt->fast, bt->nblk, bt->smem, bt->stream, bt->d_reps, bt->d_blkmap);
    k_md_sum_batch<<<(unsigned)bt->reps.size(), 32, 0, bt->stream>>>(bt->d_sums);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(bt->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return bcuda(bt, e, "batch capture end");
    e = cudaGraphInstantiate(&bt->gexec, graph, 0);
    cudaGraphDestroy(graph);
    return bcuda(bt, e, "batch graph instantiate");
}

extern "C" {

int pimd_batch_create(pimd_batch **out, const pimd_params *common, const pimd_replica *reps, int nrep,
                      const pimd_md_params *mp) {
    if (!out || !common || !reps || nrep < 1 || !mp) return PIMD_ERR_ARG;
    *out = nullptr;
    pimd_batch *bt = new pimd_batch();
    bt->mp = *mp;
    bt->device = common->device;
    int rc = bcuda(bt, cudaSetDevice(bt->device), "cudaSetDevice");
    // group replicas by box: same molecule count, box and cutoff
    std::map<std::tuple<int, double, double, double, double>, int> key2g;
    for (int i = 0; i < nrep && !rc; i++) {
        const pimd_replica &r = reps[i];
        if (r.natoms <= 0 || r.natoms % 3 || r.nbeads < 1 || r.nbeads > 64 || !(r.temp > 0) ||
            !(r.box[0] > 0 && r.box[1] > 0 && r.box[2] > 0)) {
            rc = bfail(bt, PIMD_ERR_ARG, "replica " + std::to_string(i) + ": natoms/nbeads/temp/box");
            break;
        }
        // the cutoff of each replica is min(rc, half its smallest box edge) (InputOutput.f90:277-281)
        const double rcr = std::min(common->rc, 0.5 * std::min(r.box[0], std::min(r.box[1], r.box[2])));
        auto key = std::make_tuple(r.natoms, r.box[0], r.box[1], r.box[2], rcr);
        auto it = key2g.find(key);
        int gi;
        if (it == key2g.end()) {
            gi = (int)bt->groups.size();
            key2g[key] = gi;
            bt->groups.emplace_back();
            bt->groups.back().natoms = r.natoms;
        } else {
            gi = it->second;
        }
        BatchGroup &g = bt->groups[gi];
        BatchReplica br;
        br.group = gi;
        br.local = (int)g.reps.size();
        br.bead0 = g.Ptot;
        br.P = r.nbeads;
        br.natoms = r.natoms;
        br.temp = r.temp;
        br.box0 = r.box[0];
        br.seed = mp->seed + (unsigned long long)i;
        g.reps.push_back(i);
        g.Ptot += r.nbeads;
        bt->reps.push_back(br);
    }
    if (!rc) rc = bcuda(bt, cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking), "stream");
    if (!rc) rc = bcuda(bt, cudaEventCreateWithFlags(&bt->ev_fork, cudaEventDisableTiming), "event");
    if (!rc) rc = balloc(bt, &bt->d_out4, 4 * (size_t)nrep);
    if (!rc) rc = balloc(bt, &bt->d_uk, (size_t)nrep);
    for (size_t gi = 0; gi < bt->groups.size() && !rc; gi++) {
        BatchGroup &g = bt->groups[gi];
        const pimd_replica &r0 = reps[g.reps[0]];
        pimd_params p = *common;
        p.natoms = g.natoms;
        p.nbeads = g.Ptot;
        for (int c = 0; c < 3; c++) p.box[c] = r0.box[c];
        const double rcr = std::min(common->rc, 0.5 * std::min(r0.box[0], std::min(r0.box[1], r0.box[2])));
        p.rc1 = rcr * (common->rc1 / common->rc);
        p.rc = rcr;
        std::vector<int> brep(g.Ptot);
        for (int ri : g.reps) {
            const BatchReplica &r = bt->reps[ri];
            for (int j = 0; j < r.P; j++) brep[r.bead0 + j] = r.local;
        }
        g.ctx = new pimd_ctx();
        rc = create_context(g.ctx->E, &p, (int)g.reps.size(), brep.data());
        if (rc) {
            bt->err = "group " + std::to_string(gi) + ": " + g.ctx->E.last_error;
            break;
        }
        g.ctx->check_every = 0;
        const size_t n = (size_t)g.Ptot * g.natoms * 3;
        if ((rc = balloc(bt, &g.RRt, n)) || (rc = balloc(bt, &g.PPt, n)) || (rc = balloc(bt, &g.dRRt, n)) ||
            (rc = balloc(bt, &g.RRc, g.reps.size() * (size_t)g.natoms * 3)))
            break;
        Engine &E = g.ctx->E;
        E.kp.RRt = g.RRt;
        E.kp.RRc = g.RRc;
        E.kp.dRRt = g.dRRt;
        cudaEvent_t ev;
        if ((rc = bcuda(bt, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event"))) break;
        bt->ev_join.push_back(ev);
    }
    // per replica: InitNormalModes (NormalModes.f90:68-218) and Init_Langevin_NM (Langevin.f90:68-98)
    for (size_t i = 0; i < bt->reps.size() && !rc; i++) {
        BatchReplica &r = bt->reps[i];
        const double omegan = KB_AMU * r.temp * r.P / HBAR;
        std::vector<double> a11, a12, a21, a22, om, ms, C;
        nm_init_host(r.P, omegan, mp->delt, 0.0, a11, a12, a21, a22, om, ms, C);
        std::vector<double> A(7 * r.P);
        for (int j = 0; j < r.P; j++) {
            A[j] = a11[j];
            A[r.P + j] = a12[j];
            A[2 * r.P + j] = a21[j];
            A[3 * r.P + j] = a22[j];
            A[4 * r.P + j] = ms[j];
            const double gammak = (j == 0) ? 0.0 : 2 * om[j];
            const double c1 = std::exp(-(mp->delt / 2.0) * gammak);
            A[5 * r.P + j] = c1;
            A[6 * r.P + j] = std::sqrt(KB_AMU * r.P * r.temp) * std::sqrt(1 - c1 * c1);
        }
        nm_extend_A(A, r.P, om);
        std::vector<double> CP;
        nm_pair_copy(C, CP);  // C, then its FP32 pairs for the mixed engine's transforms
        if ((rc = balloc(bt, &r.d_C, CP.size())) || (rc = balloc(bt, &r.d_A, A.size()))) break;
        cudaMemcpy(r.d_C, CP.data(), sizeof(double) * CP.size(), cudaMemcpyHostToDevice);
        nm_smem_optin(r.P);
        cudaMemcpy(r.d_A, A.data(), sizeof(double) * A.size(), cudaMemcpyHostToDevice);
    }
    // the tables of the batched integrator launches (k_md_batch, k_md_sum_batch)
    if (!rc) {
        std::vector<NMBatchRep> hr(bt->reps.size());
        std::vector<NMSumRep> hs(bt->reps.size());
        std::vector<int2> map;
        for (size_t i = 0; i < bt->reps.size(); i++) {
            const BatchReplica &r = bt->reps[i];
            BatchGroup &g = bt->groups[r.group];
            Engine &E = g.ctx->E;
            const size_t na3 = (size_t)r.natoms * 3;
            NMArgs a = replica_args(bt, r, E);
            if (a.fast) nm_fast_args(a);
            bt->fast = a.fast != 0;
            hr[i] = NMBatchRep{a, g.RRt + r.bead0 * na3, g.PPt + r.bead0 * na3, g.dRRt + r.bead0 * na3, g.RRc + r.local * na3,
                               bt->d_uk + i};
            double *d = E.d_out;
            hs[i] = NMSumRep{r.P, d + r.bead0, d + g.Ptot + r.bead0, d + 2 * g.Ptot + r.bead0, bt->d_uk + i, bt->d_out4 + 4 * i};
            const int G = std::max(1, 256 / (3 * r.P));  // atoms per block of 256 threads
            const int nb = (r.natoms + G - 1) / G;
            for (int k = 0; k < nb; k++) map.push_back(make_int2((int)i, k));
            const size_t sm = a.fast ? nm_fast_smem(r.P, G) : sizeof(double) * ((size_t)(r.P + 1) * r.P + (size_t)G * 9 * r.P);
            bt->smem = std::max(bt->smem, sm);
        }
        bt->nblk = (int)map.size();
        if ((rc = balloc(bt, &bt->d_reps, hr.size())) || (rc = balloc(bt, &bt->d_blkmap, map.size())) ||
            (rc = balloc(bt, &bt->d_sums, hs.size())))
            ;
        else {
            cudaMemcpy(bt->d_reps, hr.data(), sizeof(NMBatchRep) * hr.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(bt->d_blkmap, map.data(), sizeof(int2) * map.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(bt->d_sums, hs.data(), sizeof(NMSumRep) * hs.size(), cudaMemcpyHostToDevice);
            nm_launch_md_batch(0, bt->fast, 0, bt->smem, bt->stream, nullptr, nullptr);  // the opt-in
        }
    }
    if (!rc) rc = bcuda(bt, cudaDeviceSynchronize(), "batch set-up");
    if (rc) {
        fprintf(stderr, "pimd_batch_create: %s\n", bt->err.c_str());
        pimd_batch_destroy(bt);
        return rc;
    }
    *out = bt;
    return PIMD_OK;
}

int pimd_batch_destroy(pimd_batch *bt) {
    if (!bt) return PIMD_OK;
    cudaSetDevice(bt->device);
    if (bt->stream) cudaStreamSynchronize(bt->stream);
    if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
    for (BatchGroup &g : bt->groups)
        if (g.ctx) pimd_destroy(g.ctx);
    for (void *p : bt->allocs) cudaFree(p);
    for (cudaEvent_t e : bt->ev_join) cudaEventDestroy(e);
    if (bt->ev_fork) cudaEventDestroy(bt->ev_fork);
    if (bt->stream) cudaStreamDestroy(bt->stream);
    delete bt;
    return PIMD_OK;
}

const char *pimd_batch_last_error(pimd_batch *bt) { return bt ? bt->err.c_str() : "null batch"; }

int pimd_batch_info(pimd_batch *bt, int *ngroups, int *group_of_replica) {
    if (!bt) return PIMD_ERR_ARG;
    if (ngroups) *ngroups = (int)bt->groups.size();
    if (group_of_replica)
        for (size_t i = 0; i < bt->reps.size(); i++) group_of_replica[i] = bt->reps[i].group;
    return PIMD_OK;
}

int pimd_batch_set_state(pimd_batch *bt, int r, const double *RRt, const double *PPt) {
    if (!bt || r < 0 || r >= (int)bt->reps.size() || !RRt || !PPt) return PIMD_ERR_ARG;
    cudaSetDevice(bt->device);
    const BatchReplica &br = bt->reps[r];
    BatchGroup &g = bt->groups[br.group];
    const size_t na3 = (size_t)br.natoms * 3, n = (size_t)br.P * na3;
    std::vector<double> rc(na3, 0.0);
    for (int j = 0; j < br.P; j++)
        for (size_t i = 0; i < na3; i++) rc[i] += RRt[j * na3 + i];
    for (size_t i = 0; i < na3; i++) rc[i] /= br.P;
    cudaMemcpy(g.RRt + br.bead0 * na3, RRt, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(g.PPt + br.bead0 * na3, PPt, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(g.RRc + br.local * na3, rc.data(), sizeof(double) * na3, cudaMemcpyHostToDevice);
    return bcuda(bt, cudaGetLastError(), "set_state");
}

int pimd_batch_get_state(pimd_batch *bt, int r, double *RRt, double *PPt, double *dRRt, double *out4) {
    if (!bt || r < 0 || r >= (int)bt->reps.size()) return PIMD_ERR_ARG;
    cudaSetDevice(bt->device);
    const BatchReplica &br = bt->reps[r];
    BatchGroup &g = bt->groups[br.group];
    const size_t na3 = (size_t)br.natoms * 3, n = (size_t)br.P * na3;
    cudaStreamSynchronize(bt->stream);
    if (RRt) cudaMemcpy(RRt, g.RRt + br.bead0 * na3, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (PPt) cudaMemcpy(PPt, g.PPt + br.bead0 * na3, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (dRRt) cudaMemcpy(dRRt, g.dRRt + br.bead0 * na3, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (out4) cudaMemcpy(out4, bt->d_out4 + 4 * (size_t)r, sizeof(double) * 4, cudaMemcpyDeviceToHost);
    return bcuda(bt, cudaGetLastError(), "get_state");
}

// Gradients of the current positions for every replica (the force call before the first step).
int pimd_batch_forces(pimd_batch *bt) {
    if (!bt) return PIMD_ERR_ARG;
    cudaSetDevice(bt->device);
    for (BatchGroup &g : bt->groups) {
        Engine &E = g.ctx->E;
        double *d = E.d_out;
        int rc = run_forces(E, 0, 1, d, d + g.Ptot, d + 2 * g.Ptot, nullptr);
        if (rc) return bfail(bt, rc, E.last_error);
        cudaError_t e = cudaStreamSynchronize(E.stream);
        if (e != cudaSuccess) return bcuda(bt, e, "batch forces");
    }
    return PIMD_OK;
}

// nsteps PIMD_VV steps of every replica, each one launch of the captured batch graph.
int pimd_batch_step(pimd_batch *bt, int nsteps) {
    if (!bt || nsteps < 0) return PIMD_ERR_ARG;
    cudaSetDevice(bt->device);
    if (!bt->gexec) {
        int rc = capture_batch(bt);
        if (rc) return rc;
    }
    for (int k = 0; k < nsteps; k++) {
        bt->t++;
        for (BatchGroup &g : bt->groups) k_set_step<<<1, 32, 0, bt->stream>>>(g.ctx->E.kp.dstep, bt->t);
        cudaError_t e = cudaGraphLaunch(bt->gexec, bt->stream);
        if (e != cudaSuccess) return bcuda(bt, e, "batch graph launch");
    }
    return bcuda(bt, cudaGetLastError(), "batch step");
}

int pimd_batch_sync(pimd_batch *bt) {
    if (!bt) return PIMD_ERR_ARG;
    cudaSetDevice(bt->device);
    return bcuda(bt, cudaStreamSynchronize(bt->stream), "batch sync");
}

// Tune the tile shapes of every group's context (pimd_autotune) on its current positions.
int pimd_batch_autotune(pimd_batch *bt) {
    if (!bt) return PIMD_ERR_ARG;
    if (bt->gexec) return bfail(bt, PIMD_ERR_STATE, "autotune before the first batch step");
    for (BatchGroup &g : bt->groups) {
        int rc = pimd_autotune(g.ctx, nullptr, nullptr);
        if (rc) return bfail(bt, rc, g.ctx->E.last_error);
    }
    return PIMD_OK;
}

}  // extern "C"
