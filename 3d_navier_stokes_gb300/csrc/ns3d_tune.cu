// ns3d_tune.cu — the autotuner and the engine factories that consult it.
//
// A grid size's FP32 engine exists in several compiled shapes: variants of the
// strided x and y passes (pencil widths TileVar<V>, x-pass radix plan
// PlansV<N, V>) and two
// z-pass forms (the persistent bulk-copy line kernel, or the CTA-synchronous
// pass). ns3d_autotune times each shape on the caller's configuration and
// keeps the fastest in a process-wide table keyed by (N, precision);
// ns3d_create and ns3d_ensemble_create build every engine in the shape the
// table holds (default: variant 0, line kernel). The table can be saved to
// and loaded from a text file (one "N precision variant zform ms" line per
// entry); NS3D_TUNING_FILE names a file loaded before the first engine is
// built.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "ns3d_base.h"
#include "ns3d_ctx.h"

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, ns3d_tuning> g_table;
bool g_env_loaded = false;
thread_local int t_force_variant = -1, t_force_zform = -1;   // set while the tuner builds a candidate

ns3d_status load_file(const char* path) {
    FILE* f = fopen(path, "r");
    if (!f) return NS3D_ERR_INVALID;
    char line[256];
    ns3d_status st = NS3D_OK;
    while (fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        ns3d_tuning t{};
        if (sscanf(line, "%d %d %d %d %f", &t.N, &t.precision, &t.variant, &t.zform, &t.ms_per_step) != 5 ||
            t.variant < 0 || t.variant >= ns3d::kTileVariants || t.zform < 0 || t.zform > 2) {
            st = NS3D_ERR_INVALID;
            continue;
        }
        g_table[{t.N, t.precision}] = t;
    }
    fclose(f);
    return st;
}

void load_env_once() {
    if (g_env_loaded) return;
    g_env_loaded = true;
    const char* p = getenv("NS3D_TUNING_FILE");
    if (p && *p) load_file(p);
}

void shape_for(int N, int prec, int* variant, int* zform) {
    if (t_force_variant >= 0) {
        *variant = t_force_variant;
        *zform = t_force_zform;
        return;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    load_env_once();
    auto it = g_table.find({N, prec});
    *variant = it == g_table.end() ? 0 : it->second.variant;
    *zform = it == g_table.end() ? 0 : it->second.zform;
}
}  // namespace

namespace ns3d {
Base* make_f32(int N, const ns3d_params* ps, int M, cudaStream_t s) {
    int v = 0, z = 0;
    shape_for(N, NS3D_FP32, &v, &z);
    Base* b = v == 1   ? make_f32_v1(N, ps, M, s)
              : v == 2 ? make_f32_v2(N, ps, M, s)
              : v == 3 ? (N >= 1024 ? make_f32_v3_large(N, ps, M, s) : make_f32_v3(N, ps, M, s))
              : v == 4 ? make_f32_v4(N, ps, M, s)
              : v == 5 ? make_f32_v5(N, ps, M, s)
              : v == 6 ? make_f32_v6(N, ps, M, s)
                       : nullptr;
    if (!b) b = make_f32_v0(N, ps, M, s);
    if (b) b->set_zform(z);
    return b;
}
Base* make_f64(int N, const ns3d_params* ps, int M, cudaStream_t s) { return make_f64_v0(N, ps, M, s); }
}  // namespace ns3d

extern "C" {

ns3d_status ns3d_autotune(const ns3d_params* params, int steps, ns3d_tuning* best, ns3d_tuning* tried, int max_tried,
                          int* n_tried) {
    if (!params || steps <= 0) return NS3D_ERR_INVALID;
    if (!ns3d::supported_n(params->N)) return NS3D_ERR_UNSUPPORTED;
    const int nvar = params->precision == NS3D_FP32 ? ns3d::kTileVariants : 1;
    ns3d_tuning win{};
    win.ms_per_step = INFINITY;
    int count = 0;
    ns3d_status last = NS3D_OK;
    for (int v = 0; v < nvar; ++v) {
        for (int z = 0; z < 3; ++z) {
            if (z == 2 && !ns3d::zgemm_size(params->N, params->precision)) continue;
            t_force_variant = v;
            t_force_zform = z;
            ns3d_ctx* c = nullptr;
            ns3d_status st = ns3d_create(params, &c);
            t_force_variant = t_force_zform = -1;
            if (st != NS3D_OK) {
                last = st;
                continue;
            }
            // skip shapes that this size does not have (fell back to another one)
            if (c->impl->variant() != v || c->impl->zform() != z) {
                ns3d_destroy(c);
                continue;
            }
            float ms = 0.f;
            st = ns3d_initial_condition(c, "SPECTRUM", 0, 4.0, 1.0);
            if (st == NS3D_OK) st = ns3d_step(c, 3);
            if (st == NS3D_OK) st = ns3d_step(c, steps);
            if (st == NS3D_OK) st = ns3d_last_step_ms(c, &ms);
            ns3d_destroy(c);
            if (st != NS3D_OK) {
                last = st;
                continue;
            }
            ns3d_tuning t{params->N, params->precision, v, z, ms / (float)steps};
            if (tried && count < max_tried) tried[count] = t;
            ++count;
            if (t.ms_per_step < win.ms_per_step) win = t;
        }
    }
    if (n_tried) *n_tried = count;
    if (count == 0) return last != NS3D_OK ? last : NS3D_ERR_UNSUPPORTED;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_table[{win.N, win.precision}] = win;
    }
    if (best) *best = win;
    return NS3D_OK;
}

ns3d_status ns3d_autotune_ensemble(const ns3d_params* members, int count, int steps, ns3d_tuning* best, int max_best,
                                   int* n_best) {
    if (!members || count <= 0 || steps <= 0) return NS3D_ERR_INVALID;
    // the (N, precision) groups of the ensemble, tuned one at a time with all of their members
    std::map<std::pair<int, int>, std::vector<ns3d_params>> groups;
    for (int i = 0; i < count; ++i) groups[{members[i].N, members[i].precision}].push_back(members[i]);
    int ng = 0;
    for (const auto& g : groups) {
        const int nvar = g.first.second == NS3D_FP32 ? ns3d::kTileVariants : 1;
        ns3d_tuning win{};
        win.ms_per_step = INFINITY;
        ns3d_status last = NS3D_ERR_UNSUPPORTED;
        for (int v = 0; v < nvar; ++v) {
            for (int z = 0; z < 3; ++z) {
                if (z == 2 && !ns3d::zgemm_size(g.first.first, g.first.second)) continue;
                // build this group's engines in shape (v, z); skip shapes the size does not have
                ns3d_params probe = g.second[0];
                t_force_variant = v;
                t_force_zform = z;
                ns3d_ctx* c = nullptr;
                ns3d_status st = ns3d_create(&probe, &c);
                const bool has = st == NS3D_OK && c->impl->variant() == v && c->impl->zform() == z;
                if (c) ns3d_destroy(c);
                ns3d_ensemble* e = nullptr;
                if (has) st = ns3d_ensemble_create(g.second.data(), (int)g.second.size(), &e);
                t_force_variant = t_force_zform = -1;
                if (!has || st != NS3D_OK) {
                    if (st != NS3D_OK) last = st;
                    continue;
                }
                for (int m = 0; m < (int)g.second.size() && st == NS3D_OK; ++m)
                    st = ns3d_ensemble_initial_condition(e, m, "SPECTRUM", (uint64_t)m, 4.0, 1.0);
                float ms = 0.f;
                if (st == NS3D_OK) st = ns3d_ensemble_step(e, 3);
                if (st == NS3D_OK) st = ns3d_ensemble_step(e, steps);
                if (st == NS3D_OK) st = ns3d_ensemble_last_step_ms(e, &ms);
                ns3d_ensemble_destroy(e);
                if (st != NS3D_OK) {
                    last = st;
                    continue;
                }
                if (ms / steps < win.ms_per_step) win = ns3d_tuning{g.first.first, g.first.second, v, z, ms / steps};
            }
        }
        if (!(win.ms_per_step < INFINITY)) return last;
        {
            std::lock_guard<std::mutex> lk(g_mu);
            g_table[{win.N, win.precision}] = win;
        }
        if (best && ng < max_best) best[ng] = win;
        ++ng;
    }
    if (n_best) *n_best = ng;
    return NS3D_OK;
}

ns3d_status ns3d_tuning_get(int N, int precision, ns3d_tuning* t) {
    if (!t) return NS3D_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    load_env_once();
    auto it = g_table.find({N, precision});
    if (it == g_table.end()) return NS3D_ERR_INVALID;
    *t = it->second;
    return NS3D_OK;
}

ns3d_status ns3d_tuning_set(const ns3d_tuning* t) {
    if (!t || t->variant < 0 || t->variant >= ns3d::kTileVariants || t->zform < 0 || t->zform > 2 ||
        (t->precision != NS3D_FP32 && t->precision != NS3D_FP64))
        return NS3D_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    g_table[{t->N, t->precision}] = *t;
    return NS3D_OK;
}

ns3d_status ns3d_tuning_clear(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.clear();
    g_env_loaded = true;
    return NS3D_OK;
}

ns3d_status ns3d_tuning_save(const char* path) {
    if (!path) return NS3D_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    FILE* f = fopen(path, "w");
    if (!f) return NS3D_ERR_INVALID;
    fprintf(f, "# N precision variant zform ms_per_step\n");
    for (const auto& kv : g_table)
        fprintf(f, "%d %d %d %d %.6f\n", kv.second.N, kv.second.precision, kv.second.variant, kv.second.zform,
                kv.second.ms_per_step);
    fclose(f);
    return NS3D_OK;
}

ns3d_status ns3d_tuning_load(const char* path) {
    if (!path) return NS3D_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    g_env_loaded = true;
    return load_file(path);
}

}  // extern "C"
