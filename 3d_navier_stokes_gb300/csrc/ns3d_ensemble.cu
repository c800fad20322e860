// ns3d_ensemble.cu — many independent runs stepped together (include/ns3d.h,
// ns3d_ensemble_*).
//
// Members that share grid size, precision, integrator, viscosity power,
// forcing and whether the CFL step is on form one group: one engine whose
// kernels cover every member of the group in the same launches (member index
// in blockIdx.z / the z pass's work list), each member with its own state,
// viscosity, time step and clock. The groups run on their own streams, and a
// whole ensemble step is captured once as a CUDA graph in which the groups'
// steps follow one another (each pass kernel of a group fills the GPU; with
// the groups as parallel branches their kernels shared the SMs and the step
// took 5.34-5.56 ms instead of 4.98 ms for the 96-member ensemble), so one
// graph launch advances every member by one step.
// ns3d_ensemble_run wraps that step in a device-side loop: a graph whose only
// top-level node is a conditional WHILE node with the step as its body and a
// one-thread kernel that counts the steps down and clears the condition at
// zero, so a whole run of n steps is a single graph launch.
#include <map>
#include <string.h>
#include <tuple>
#include <vector>

#include "ns3d_base.h"

namespace ns3d {
ns3d_status ic_dispatch(Base* impl, int N, const char* name, uint64_t seed, double k0, double energy);
}

struct ns3d_ensemble {
    std::vector<ns3d::Base*> groups;
    std::vector<cudaStream_t> streams;
    std::vector<int> group_n;
    std::vector<std::pair<int, int>> where;   // member -> (group, index in the group)
    cudaStream_t main = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t loop = nullptr;            // the step in a device-side while loop
    long long* d_count = nullptr;              // steps left in the loop
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    char err[512] = {0};
};

static ns3d_status ens_fail(ns3d_ensemble* e, ns3d_status s, const char* msg) {
    if (e) snprintf(e->err, sizeof(e->err), "%s", msg);
    return s;
}

static void ens_free(ns3d_ensemble* e) {
    if (!e) return;
    if (e->main) cudaStreamSynchronize(e->main);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    if (e->loop) cudaGraphExecDestroy(e->loop);
    if (e->d_count) cudaFree(e->d_count);
    for (auto* g : e->groups) delete g;
    for (auto s : e->streams) cudaStreamDestroy(s);
    if (e->main) cudaStreamDestroy(e->main);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    delete e;
}

static ns3d_status ens_member(ns3d_ensemble* e, int m, ns3d::Base** impl, int* N) {
    if (!e || m < 0 || m >= (int)e->where.size()) return NS3D_ERR_INVALID;
    const auto gw = e->where[m];
    *impl = e->groups[gw.first];
    if (N) *N = e->group_n[gw.first];
    return (*impl)->select(gw.second);
}

static ns3d_status ens_pass(ns3d_ensemble* e, ns3d::Base* impl, ns3d_status s) {
    if (s != NS3D_OK && impl) snprintf(e->err, sizeof(e->err), "%s", impl->err());
    return s;
}

// the loop body's last node: one step done; continue while steps are left
__global__ void k_loop_count(cudaGraphConditionalHandle h, long long* count) {
    const long long left = --(*count);
    cudaGraphSetConditional(h, left > 0 ? 1u : 0u);
}

// Enqueue one step of every group (forked from and joined back into main).
static cudaError_t ens_enqueue(ns3d_ensemble* e, cudaEvent_t fork, std::vector<cudaEvent_t>& join) {
    cudaError_t err = cudaEventRecord(fork, e->main);
    cudaEvent_t prev = fork;
    for (size_t i = 0; err == cudaSuccess && i < e->groups.size(); ++i) {
        err = cudaStreamWaitEvent(e->streams[i], prev, 0);
        if (err != cudaSuccess) break;
        e->groups[i]->enqueue_step();
        err = cudaEventRecord(join[i], e->streams[i]);
        prev = join[i];
    }
    if (err == cudaSuccess) err = cudaStreamWaitEvent(e->main, prev, 0);
    return err;
}

static ns3d_status ens_build_loop(ns3d_ensemble* e) {
    if (e->loop) return NS3D_OK;
    if (!e->d_count && cudaMalloc(&e->d_count, sizeof(long long)) != cudaSuccess)
        return ens_fail(e, NS3D_ERR_NOMEM, "loop counter");
    std::vector<cudaEvent_t> join(e->groups.size());
    cudaEvent_t fork;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return NS3D_ERR_CUDA;
    for (auto& j : join) cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h = 0;
    cudaGraphNode_t node = nullptr;
    cudaError_t err = cudaGraphCreate(&g, 0);
    // the condition starts at 1 on every launch; the body clears it after the last step
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    if (err == cudaSuccess) err = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    if (err == cudaSuccess) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        err = cudaStreamBeginCaptureToGraph(e->main, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
            cudaError_t e1 = ens_enqueue(e, fork, join);
            if (e1 == cudaSuccess) {
                k_loop_count<<<1, 1, 0, e->main>>>(h, e->d_count);
                e1 = cudaGetLastError();
            }
            cudaGraph_t captured = nullptr;
            err = cudaStreamEndCapture(e->main, &captured);
            if (err == cudaSuccess) err = e1;
        }
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&e->loop, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaEventDestroy(fork);
    for (auto& j : join) cudaEventDestroy(j);
    if (err != cudaSuccess) {
        e->loop = nullptr;
        cudaGetLastError();
        snprintf(e->err, sizeof(e->err), "ensemble loop graph: %s", cudaGetErrorString(err));
        return NS3D_ERR_CUDA;
    }
    return NS3D_OK;
}

static ns3d_status ens_build_graph(ns3d_ensemble* e) {
    if (e->graph) return NS3D_OK;
    std::vector<cudaEvent_t> join(e->groups.size());
    cudaEvent_t fork;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return NS3D_ERR_CUDA;
    for (auto& j : join) cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    cudaGraph_t g = nullptr;
    cudaError_t err = cudaStreamBeginCapture(e->main, cudaStreamCaptureModeThreadLocal);
    if (err == cudaSuccess) err = ens_enqueue(e, fork, join);
    cudaError_t e2 = cudaStreamEndCapture(e->main, &g);
    if (err == cudaSuccess) err = e2;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&e->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaEventDestroy(fork);
    for (auto& j : join) cudaEventDestroy(j);
    if (err != cudaSuccess) {
        e->graph = nullptr;
        snprintf(e->err, sizeof(e->err), "ensemble graph: %s", cudaGetErrorString(err));
        return NS3D_ERR_CUDA;
    }
    return NS3D_OK;
}

extern "C" {

ns3d_status ns3d_ensemble_create(const ns3d_params* members, int count, ns3d_ensemble** out) {
    if (!members || count <= 0 || !out) return NS3D_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < count; ++i) {
        const ns3d_params* p = &members[i];
        if (p->N <= 2 || (p->N % 2) || !(p->nu > 0) || !(p->dt > 0) || p->t0 < 0) return NS3D_ERR_INVALID;
        if (!ns3d::supported_n(p->N)) return NS3D_ERR_UNSUPPORTED;
        if ((p->visc_pow != 1 && p->visc_pow != 2) || (p->integrator < NS3D_IFRK4 || p->integrator > NS3D_RK5CN) ||
            (p->precision != NS3D_FP64 && p->precision != NS3D_FP32) || p->cfl < 0 ||
            (p->forcing != NS3D_FORCE_NONE && p->forcing != NS3D_FORCE_SHELL) ||
            (p->forcing == NS3D_FORCE_SHELL && (p->force_k < 1 || p->force_k > p->N / 3)) ||
            p->device != members[0].device)
            return NS3D_ERR_INVALID;
    }
    if (cudaSetDevice(members[0].device) != cudaSuccess) return NS3D_ERR_CUDA;
    // group members by everything that is a template or launch-wide switch
    typedef std::tuple<int, int, int, int, int, int, int> key_t;
    std::map<key_t, std::vector<int>> by;
    for (int i = 0; i < count; ++i) {
        const ns3d_params& p = members[i];
        by[key_t(p.N, p.precision, p.integrator, p.visc_pow, p.forcing, p.forcing ? p.force_k : 0, p.cfl > 0)]
            .push_back(i);
    }
    ns3d_ensemble* e = new ns3d_ensemble();
    e->where.resize(count);
    if (cudaStreamCreateWithFlags(&e->main, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess) {
        ens_free(e);
        return NS3D_ERR_CUDA;
    }
    for (auto& kv : by) {
        std::vector<ns3d_params> ps;
        for (int i : kv.second) ps.push_back(members[i]);
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            ens_free(e);
            return NS3D_ERR_CUDA;
        }
        e->streams.push_back(s);
        const int N = ps[0].N;
        ns3d::Base* g = ps[0].precision == NS3D_FP32 ? ns3d::make_f32(N, ps.data(), (int)ps.size(), s)
                                                     : ns3d::make_f64(N, ps.data(), (int)ps.size(), s);
        if (!g) {
            ens_free(e);
            return NS3D_ERR_UNSUPPORTED;
        }
        e->groups.push_back(g);
        e->group_n.push_back(N);
        const ns3d_status st = g->init();
        if (st != NS3D_OK) {
            const bool oom = strstr(g->err(), "out of memory") != nullptr;
            ens_free(e);
            cudaGetLastError();
            return oom ? NS3D_ERR_NOMEM : st;
        }
        for (size_t j = 0; j < kv.second.size(); ++j)
            e->where[kv.second[j]] = std::make_pair((int)e->groups.size() - 1, (int)j);
    }
    *out = e;
    return NS3D_OK;
}

ns3d_status ns3d_ensemble_destroy(ns3d_ensemble* e) {
    if (!e) return NS3D_ERR_INVALID;
    ens_free(e);
    return NS3D_OK;
}

const char* ns3d_ensemble_last_error(const ns3d_ensemble* e) { return e ? e->err : "null ensemble"; }

ns3d_status ns3d_ensemble_initial_condition(ns3d_ensemble* e, int member, const char* name, uint64_t seed, double k0,
                                            double energy) {
    ns3d::Base* g = nullptr;
    int N = 0;
    ns3d_status s = ens_member(e, member, &g, &N);
    if (s != NS3D_OK) return s;
    if (!name) return NS3D_ERR_INVALID;
    return ens_pass(e, g, ns3d::ic_dispatch(g, N, name, seed, k0, energy));
}

ns3d_status ns3d_ensemble_set_state_host(ns3d_ensemble* e, int member, const double* u_hat) {
    ns3d::Base* g = nullptr;
    ns3d_status s = ens_member(e, member, &g, nullptr);
    if (s != NS3D_OK || !u_hat) return s != NS3D_OK ? s : NS3D_ERR_INVALID;
    return ens_pass(e, g, g->set_state_host(u_hat));
}

ns3d_status ns3d_ensemble_get_state_host(ns3d_ensemble* e, int member, double* u_hat) {
    ns3d::Base* g = nullptr;
    ns3d_status s = ens_member(e, member, &g, nullptr);
    if (s != NS3D_OK || !u_hat) return s != NS3D_OK ? s : NS3D_ERR_INVALID;
    return ens_pass(e, g, g->get_state_host(u_hat));
}

ns3d_status ns3d_ensemble_measurables(ns3d_ensemble* e, int member, ns3d_measures* m, double* Ek, double* Ok) {
    ns3d::Base* g = nullptr;
    ns3d_status s = ens_member(e, member, &g, nullptr);
    if (s != NS3D_OK) return s;
    return ens_pass(e, g, g->measurables(m, Ek, Ok));
}

ns3d_status ns3d_ensemble_get_time(ns3d_ensemble* e, int member, double* t, double* dt, long* iters) {
    ns3d::Base* g = nullptr;
    ns3d_status s = ens_member(e, member, &g, nullptr);
    if (s != NS3D_OK) return s;
    return ens_pass(e, g, g->get_time(t, dt, iters));
}

ns3d_status ns3d_ensemble_step(ns3d_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return NS3D_ERR_INVALID;
    if (nsteps == 0) return NS3D_OK;
    // outstanding work on the group streams (initial conditions) precedes the graph
    for (auto s : e->streams)
        if (cudaStreamSynchronize(s) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "group stream failed");
    ns3d_status st = ens_build_graph(e);
    if (st != NS3D_OK) return st;
    if (cudaEventRecord(e->ev0, e->main) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "event record");
    for (int k = 0; k < nsteps; ++k)
        if (cudaGraphLaunch(e->graph, e->main) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "graph launch");
    if (cudaEventRecord(e->ev1, e->main) != cudaSuccess || cudaStreamSynchronize(e->main) != cudaSuccess)
        return ens_fail(e, NS3D_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    for (auto* g : e->groups) {
        st = g->status();
        if (st != NS3D_OK) return ens_pass(e, g, st);
    }
    return NS3D_OK;
}

ns3d_status ns3d_ensemble_run(ns3d_ensemble* e, int nsteps) {
    if (!e || nsteps < 0) return NS3D_ERR_INVALID;
    if (nsteps == 0) return NS3D_OK;
    for (auto s : e->streams)
        if (cudaStreamSynchronize(s) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "group stream failed");
    ns3d_status st = ens_build_loop(e);
    if (st != NS3D_OK) return st;
    const long long n = nsteps;
    if (cudaMemcpyAsync(e->d_count, &n, sizeof(n), cudaMemcpyHostToDevice, e->main) != cudaSuccess)
        return ens_fail(e, NS3D_ERR_CUDA, "loop counter");
    if (cudaEventRecord(e->ev0, e->main) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "event record");
    if (cudaGraphLaunch(e->loop, e->main) != cudaSuccess) return ens_fail(e, NS3D_ERR_CUDA, "loop graph launch");
    if (cudaEventRecord(e->ev1, e->main) != cudaSuccess || cudaStreamSynchronize(e->main) != cudaSuccess)
        return ens_fail(e, NS3D_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    for (auto* g : e->groups) {
        st = g->status();
        if (st != NS3D_OK) return ens_pass(e, g, st);
    }
    return NS3D_OK;
}

ns3d_status ns3d_ensemble_info(ns3d_ensemble* e, int* groups, int* kernels_per_step) {
    if (!e) return NS3D_ERR_INVALID;
    if (groups) *groups = (int)e->groups.size();
    if (kernels_per_step) {
        int k = 0;
        for (auto* g : e->groups) k += g->kernels_per_step();
        *kernels_per_step = k;
    }
    return NS3D_OK;
}

ns3d_status ns3d_ensemble_last_step_ms(ns3d_ensemble* e, float* ms) {
    if (!e || !ms) return NS3D_ERR_INVALID;
    return cudaEventElapsedTime(ms, e->ev0, e->ev1) == cudaSuccess ? NS3D_OK : NS3D_ERR_CUDA;
}

ns3d_status ns3d_ensemble_profile(ns3d_ensemble* e, int group, int reps, const char** names, float* ms,
                                  double* bytes, int max_count, int* count, int* n_out) {
    if (!e || group < 0 || group >= (int)e->groups.size() || reps <= 0 || !names || !ms || !count)
        return NS3D_ERR_INVALID;
    if (n_out) *n_out = e->group_n[group];
    const ns3d_status st = e->groups[group]->profile(reps, names, ms, bytes, max_count, count);
    if (st != NS3D_OK) snprintf(e->err, sizeof(e->err), "%s", e->groups[group]->err());
    return st;
}

}  // extern "C"
