// nb_tune.cu -- autotuner of a handle's kernel and list shapes, and its cache.
//
// MOIL's list scheme is fixed (pot/nbondm.f:143-210, pot/nbond.f:54-157); here the same pair
// set can be evaluated with several shapes (moil_nb_shape): the number of concurrently
// evaluated replica groups, the full- or half-list water kernel and its block size, and the
// way the water rows are built (cell search or all-pairs tiles).  Which is fastest depends on
// the GPU and on the batch (replica count and sizes), so moil_nb_autotune times short runs of
// each candidate on the caller's own batch -- coordinate descent over the three knobs, every
// candidate timed over one list period of device-resident evaluations -- and keeps the
// fastest.  The result can be cached in a text file keyed by the GPU and the replica-size
// histogram; moil_nb_init_batch applies a cached shape before it builds the handle.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "nb_internal.h"

namespace {

// GPU model, multiprocessors, precision, replica count, the replica-size histogram over
// power-of-two atom-count bins, and the timed call (device-resident or host buffers)
std::string tune_key(int device, int nrep, const moil_replica *reps, int mode)
{
    cudaDeviceProp prop;
    std::string gpu = "unknown";
    int nsm = 0;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
        gpu = prop.name;
        nsm = prop.multiProcessorCount;
    }
    std::replace(gpu.begin(), gpu.end(), ' ', '_');
    int hist[32] = {0};
    for (int r = 0; r < nrep; ++r) {
        const int n = reps[r].topo ? reps[r].topo->npt : 0;
        int b = 0;
        while (b < 31 && (2 << b) <= n) ++b;
        hist[b]++;
    }
    std::ostringstream k;
    k << gpu << "|sm" << nsm << "|prec" << (nrep > 0 ? reps[0].params->precision : 0) << "|nrep" << nrep << "|hist";
    for (int b = 0; b < 32; ++b)
        if (hist[b]) k << ":" << b << "=" << hist[b];
    if (mode == MOIL_NB_TUNE_HOST) k << "|host";
    return k.str();
}

// cache lines: key <TAB> water_kernel half_block tiled groups <TAB> ms per evaluation
bool cache_lookup(const std::string &path, const std::string &key, moil_nb_shape *s)
{
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t t1 = line.find('\t');
        if (t1 == std::string::npos || line.compare(0, t1, key) != 0) continue;
        std::istringstream v(line.substr(t1 + 1));
        moil_nb_shape x{};
        if (v >> x.water_kernel >> x.half_block >> x.tiled >> x.groups) {
            *s = x;
            return true;
        }
    }
    return false;
}

bool cache_store(const std::string &path, const std::string &key, const moil_nb_shape &s, double ms)
{
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line)) {
            const size_t t1 = line.find('\t');
            if (t1 != std::string::npos && line.compare(0, t1, key) == 0) continue;
            if (!line.empty()) keep.push_back(line);
        }
    }
    std::ostringstream e;
    e << key << '\t' << s.water_kernel << ' ' << s.half_block << ' ' << s.tiled << ' ' << s.groups << '\t' << ms;
    keep.push_back(e.str());
    const std::string tmp = path + ".tmp";
    {
        std::ofstream f(tmp, std::ios::trunc);
        if (!f) return false;
        for (const std::string &l : keep) f << l << '\n';
        if (!f) return false;
    }
    return std::rename(tmp.c_str(), path.c_str()) == 0;
}

bool same_shape(const moil_nb_shape &a, const moil_nb_shape &b)
{
    return a.water_kernel == b.water_kernel && a.half_block == b.half_block && a.tiled == b.tiled &&
           a.groups == b.groups;
}

}  // namespace

// applied by moil_nb_init_batch before the handle is built (nb_host.cu)
int nb_tune_cached_shape(moil_nb_ctx *h, int nrep, const moil_replica *reps)
{
    if (h->tune_cache.empty() || h->tuning || nrep <= 0 || !reps) return 0;
    moil_nb_shape s;
    if (!cache_lookup(h->tune_cache, tune_key(h->device, nrep, reps, h->tune_mode), &s)) return 0;
    h->want_whalf = s.water_kernel;
    h->hb = s.half_block ? s.half_block : 256;
    h->want_tiled = s.tiled;
    h->want_groups = s.groups;
    return 1;
}

extern "C" {

int moil_nb_set_tune_cache(moil_nb_ctx *h, const char *path)
{
    if (!h) return MOIL_NB_ERR_ARG;
    h->tune_cache = path ? path : "";
    return MOIL_NB_OK;
}

int moil_nb_set_tune_mode(moil_nb_ctx *h, int mode)
{
    if (!h || (mode != MOIL_NB_TUNE_DEVICE && mode != MOIL_NB_TUNE_HOST)) return MOIL_NB_ERR_ARG;
    h->tune_mode = mode;
    return MOIL_NB_OK;
}

int moil_nb_autotune(moil_nb_ctx *h, int nrep, const moil_replica *reps, const double *d_coor, double *d_dpot,
                     int evals, moil_nb_shape *best, moil_nb_tune_trial *trials, int max_trials, int *ntrials)
{
    if (!h || nrep <= 0 || !reps || !d_coor || !d_dpot) return MOIL_NB_ERR_ARG;
    if (h->pending) return MOIL_NB_ERR_STATE;
    for (int r = 0; r < nrep; ++r)
        if (!reps[r].params || !reps[r].topo) return MOIL_NB_ERR_ARG;
    if (ntrials) *ntrials = 0;
    if (evals <= 0) evals = reps[0].params->list_period > 0 ? reps[0].params->list_period : 10;
    evals = std::max(evals, 3);
    // host mode: page-locked copies of the batch for moil_nb_eval (freed on every return path)
    struct Pinned {
        double *c = nullptr, *d = nullptr;
        ~Pinned() { if (c) cudaFreeHost(c); if (d) cudaFreeHost(d); }
    } hb;
    if (h->tune_mode == MOIL_NB_TUNE_HOST) {
        int64_t natom = 0;
        for (int r = 0; r < nrep; ++r) natom += reps[r].topo->npt;
        const size_t bytes = sizeof(double) * 3 * (size_t)natom;
        NB_CUDA_OK(h, cudaMallocHost(&hb.c, bytes));
        NB_CUDA_OK(h, cudaMallocHost(&hb.d, bytes));
        NB_CUDA_OK(h, cudaMemcpy(hb.c, d_coor, bytes, cudaMemcpyDeviceToHost));
    }
    auto one_eval = [&]() -> int {
        return hb.c ? moil_nb_eval(h, hb.c, hb.d, nullptr) : moil_nb_eval_device(h, d_coor, d_dpot, nullptr);
    };
    h->tuning = 1;
    std::vector<moil_nb_tune_trial> log;
    int inited_groups = -1;        // the group count the handle was last built with here
    auto measure = [&](const moil_nb_shape &s, double *ms) -> int {
        int rc = moil_nb_set_shape(h, &s);
        if (rc != MOIL_NB_OK) return rc;
        if (!h->inited || s.groups != inited_groups) {
            rc = moil_nb_init_batch(h, nrep, reps);
            if (rc != MOIL_NB_OK) return rc;
            inited_groups = s.groups;
            rc = moil_nb_set_shape(h, &s);     // in-handle shapes of the new groups
            if (rc != MOIL_NB_OK) return rc;
        }
        for (int k = 0; k < 2; ++k) {          // list build, graph capture
            rc = one_eval();
            if (rc != MOIL_NB_OK) return rc;
        }
        const auto t0 = std::chrono::steady_clock::now();
        for (int k = 0; k < evals; ++k) {
            rc = one_eval();
            if (rc != MOIL_NB_OK) return rc;
        }
        *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() / evals;
        moil_nb_tune_trial t;
        moil_nb_get_shape(h, &t.shape);
        t.shape.tiled = s.tiled;
        t.ms_per_eval = *ms;
        log.push_back(t);
        return MOIL_NB_OK;
    };
    int rc = MOIL_NB_OK;
    moil_nb_shape cur = {MOIL_NB_WATER_AUTO, 0, MOIL_NB_TILED_AUTO, 0};
    double best_ms = 1e300;
    moil_nb_shape best_s = cur;
    auto consider = [&](const moil_nb_shape &s) -> int {
        for (const moil_nb_tune_trial &t : log)
            if (same_shape(t.shape, s)) return MOIL_NB_OK;     // resolved to a shape already timed
        double ms;
        const int r = measure(s, &ms);
        if (r != MOIL_NB_OK) return r;
        moil_nb_shape got = log.back().shape;
        if (ms < best_ms) { best_ms = ms; best_s = got; }
        return MOIL_NB_OK;
    };
    // 1. replica groups (the handle is rebuilt for each)
    for (int P = 1; P <= std::min(nrep, 4) && rc == MOIL_NB_OK; ++P) {
        moil_nb_shape s = cur;
        s.groups = P;
        rc = consider(s);
    }
    // 2. water kernel: full lists, half lists in blocks of 128, 256 and 512 waters
    if (rc == MOIL_NB_OK) {
        cur = best_s;
        const moil_nb_shape cand[4] = {{MOIL_NB_WATER_FULL, 256, cur.tiled, cur.groups},
                                       {MOIL_NB_WATER_HALF, 128, cur.tiled, cur.groups},
                                       {MOIL_NB_WATER_HALF, 256, cur.tiled, cur.groups},
                                       {MOIL_NB_WATER_HALF, 512, cur.tiled, cur.groups}};
        for (int k = 0; k < 4 && rc == MOIL_NB_OK; ++k) rc = consider(cand[k]);
    }
    // 3. how the water rows are built
    if (rc == MOIL_NB_OK) {
        cur = best_s;
        for (int t = MOIL_NB_TILED_AUTO; t <= MOIL_NB_TILED_ALL && rc == MOIL_NB_OK; ++t) {
            moil_nb_shape s = cur;
            s.tiled = t;
            rc = consider(s);
        }
    }
    // the winner stays applied
    if (rc == MOIL_NB_OK) {
        rc = moil_nb_set_shape(h, &best_s);
        if (rc == MOIL_NB_OK && best_s.groups != inited_groups) {
            rc = moil_nb_init_batch(h, nrep, reps);
            if (rc == MOIL_NB_OK) rc = moil_nb_set_shape(h, &best_s);
        }
    }
    h->tuning = 0;
    if (rc != MOIL_NB_OK) return rc;
    if (!h->tune_cache.empty() &&
        !cache_store(h->tune_cache, tune_key(h->device, nrep, reps, h->tune_mode), best_s, best_ms)) {
        h->err = "moil_nb_autotune: cannot write the cache file " + h->tune_cache;
        return MOIL_NB_ERR_ARG;
    }
    if (best) *best = best_s;
    if (ntrials) *ntrials = (int)log.size();
    if (trials)
        for (int k = 0; k < (int)log.size() && k < max_trials; ++k) trials[k] = log[k];
    return MOIL_NB_OK;
}

}  // extern "C"
