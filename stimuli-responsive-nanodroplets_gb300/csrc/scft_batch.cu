/*
 * scft_batch.cu — the batching form over instances of uneven grid sizes.
 *
 * A context holds instances of one grid (they share the operator geometry,
 * the slice stride and the shape of the persistent chain kernel). A batch
 * groups its surfaces by grid, MASK, active field set and species
 * composition, gives every group its own context (own stream, own CUDA graph
 * of one iteration, persistent chain kernel over all of the group's chains),
 * and runs the groups side by side: each round enqueues a chunk of iterations
 * on every group that still has unconverged instances, then collects them.
 * The groups' kernels overlap on the device; instances that meet their stop
 * criterion are frozen on the device and cost nothing in later rounds.
 *
 * The reference runs one instance per process to a fixed ITER (SCFT.c:1088);
 * this file has no counterpart there.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

#include "scft_internal.h"

struct scft_batch {
    int n = 0;
    std::vector<scft_ctx *> ctx;            /* [groups] */
    std::vector<std::vector<int>> members;  /* [groups] -> instance indices */
    std::vector<int> group, slot;           /* [n] */
    std::vector<unsigned long> iter;        /* [n] current iIter */
    std::vector<scft_iter_out> last;        /* [n] latest record */
    std::vector<char> idle;                 /* [n] frozen (converged or scft_batch_freeze) and not
                                               re-armed since: a group of idle instances is not run */
};

/* Instances that can share a context: same grid, MASK, active fields and
 * which species are present (contour counts, lengths, chi may differ). */
static std::string group_key(const scft_surface &s, const scft_derived &d)
{
    char buf[256];
    int n = snprintf(buf, sizeof(buf), "%d,%d,%d,%d,%d|", d.nx, d.ny, d.nz, s.mask, d.n_active);
    std::string k(buf, n);
    for (int f = 0; f < 13; ++f) k += d.active[f] ? '1' : '0';
    k += '|';
    for (int i = 0; i < 4; ++i) k += s.vol_dbk[i] > 0.0 ? '1' : '0';
    for (int i = 0; i < 10; ++i) k += d.ns_homo[i] > 0 ? '1' : '0';
    for (int i = 0; i < 3; ++i) k += d.ns_s[i] > 0 ? '1' : '0';
    return k;
}

extern "C" int scft_batch_destroy(scft_batch *b)
{
    if (!b) return SCFT_OK;
    for (scft_ctx *c : b->ctx) scft_ctx_destroy(c);
    delete b;
    return SCFT_OK;
}

extern "C" int scft_batch_create(const scft_surface *surfaces, int n, const scft_options *opt, scft_batch **out)
{
    if (!surfaces || n < 1 || !out) return SCFT_ERR_PARAM;
    *out = nullptr;
    scft_batch *b = new scft_batch();
    b->n = n;
    b->group.assign(n, -1);
    b->slot.assign(n, -1);
    b->iter.assign(n, 0);
    b->last.assign(n, scft_iter_out{});
    b->idle.assign(n, 0);
    std::map<std::string, int> by_key;
    for (int i = 0; i < n; ++i) {
        scft_derived d;
        int rc = scft_derive(&surfaces[i], &d);
        if (rc != SCFT_OK) {
            char msg[128];
            snprintf(msg, sizeof(msg), "batch instance %d: parameter derivation failed (%d)", i, rc);
            scft_set_error(msg);
            scft_batch_destroy(b);
            return rc;
        }
        const std::string k = group_key(surfaces[i], d);
        auto it = by_key.find(k);
        int g;
        if (it == by_key.end()) {
            g = (int)b->members.size();
            by_key[k] = g;
            b->members.emplace_back();
        } else {
            g = it->second;
        }
        b->group[i] = g;
        b->slot[i] = (int)b->members[g].size();
        b->members[g].push_back(i);
    }
    scft_options o;
    if (opt)
        o = *opt;
    else
        scft_options_default(&o);
    for (size_t g = 0; g < b->members.size(); ++g) {
        std::vector<scft_surface> s;
        for (int i : b->members[g]) s.push_back(surfaces[i]);
        o.n_instances = (int)s.size();
        scft_ctx *c = nullptr;
        int rc = scft_ctx_create(s.data(), &o, &c);
        if (rc != SCFT_OK) {
            scft_batch_destroy(b);
            return rc;
        }
        b->ctx.push_back(c);
    }
    *out = b;
    return SCFT_OK;
}

extern "C" int scft_batch_groups(const scft_batch *b) { return b ? (int)b->ctx.size() : 0; }

extern "C" int scft_batch_locate(const scft_batch *b, int i, int *group, int *slot)
{
    if (!b || i < 0 || i >= b->n) return SCFT_ERR_PARAM;
    if (group) *group = b->group[i];
    if (slot) *slot = b->slot[i];
    return SCFT_OK;
}

extern "C" scft_ctx *scft_batch_context(scft_batch *b, int group)
{
    if (!b || group < 0 || group >= (int)b->ctx.size()) return nullptr;
    return b->ctx[group];
}

#define LOCATE(b, i)                                               \
    if (!(b) || (i) < 0 || (i) >= (b)->n) return SCFT_ERR_PARAM;   \
    scft_ctx *c_ = (b)->ctx[(b)->group[i]];                        \
    const int s_ = (b)->slot[i]

extern "C" int scft_batch_set_fields(scft_batch *b, int i, const double *w14)
{
    LOCATE(b, i);
    return scft_set_fields(c_, s_, w14);
}

extern "C" int scft_batch_set_masks(scft_batch *b, int i, const double *mask3)
{
    LOCATE(b, i);
    return scft_set_masks(c_, s_, mask3);
}

extern "C" int scft_batch_set_iteration(scft_batch *b, int i, unsigned long it)
{
    LOCATE(b, i);
    int rc = scft_set_iteration(c_, s_, it);
    if (rc == SCFT_OK) {
        b->iter[i] = it;
        b->idle[i] = 0; /* re-armed */
    }
    return rc;
}

extern "C" int scft_batch_set_rng(scft_batch *b, int i, const unsigned short seed[3])
{
    LOCATE(b, i);
    return scft_set_rng(c_, s_, seed);
}

extern "C" int scft_batch_set_stop(scft_batch *b, int i, double rms_tol)
{
    LOCATE(b, i);
    return scft_set_stop(c_, s_, rms_tol);
}

extern "C" int scft_batch_freeze(scft_batch *b, int i)
{
    LOCATE(b, i);
    int rc = scft_freeze(c_, s_);
    if (rc == SCFT_OK) b->idle[i] = 1;
    return rc;
}

extern "C" int scft_batch_get_fields(scft_batch *b, int i, double *w14)
{
    LOCATE(b, i);
    return scft_get_fields(c_, s_, w14);
}

extern "C" int scft_batch_get_densities(scft_batch *b, int i, double *phi13, double *phi_tot)
{
    LOCATE(b, i);
    return scft_get_densities(c_, s_, phi13, phi_tot);
}

/* Run every instance until it converges (scft_batch_set_stop) or has run
 * max_iter iterations in this call; chunk iterations per group per round
 * (<= SCFT_HIST_CAP). res[i] gets the iterations run in this call, the last
 * record's free energy, RMS, convergence flag and status. */
extern "C" int scft_batch_run(scft_batch *b, int max_iter, int chunk, scft_batch_result *res)
{
    if (!b || max_iter < 0 || chunk < 1 || chunk > SCFT_HIST_CAP) return SCFT_ERR_PARAM;
    const int G = (int)b->ctx.size();
    std::vector<unsigned long> start(b->iter);
    std::vector<int> ran(G, 0), live(G, 1);
    /* a group whose instances are all frozen would only repeat their records */
    for (int g = 0; g < G; ++g) {
        int all_idle = 1;
        for (int i : b->members[g]) all_idle &= b->idle[i] ? 1 : 0;
        if (all_idle) live[g] = 0;
    }
    std::vector<std::vector<scft_iter_out>> recs(G);
    for (int g = 0; g < G; ++g) recs[g].resize((size_t)chunk * b->members[g].size());
    int status = SCFT_OK;
    for (;;) {
        std::vector<int> k(G, 0);
        int any = 0;
        for (int g = 0; g < G; ++g) {
            if (!live[g]) continue;
            k[g] = max_iter - ran[g] < chunk ? max_iter - ran[g] : chunk;
            if (k[g] <= 0) {
                live[g] = 0;
                continue;
            }
            int rc = scft_iterate_async(b->ctx[g], k[g]);
            if (rc != SCFT_OK) {
                /* collect what is already in flight before reporting */
                for (int h = 0; h < g; ++h)
                    if (k[h] > 0) scft_iterate_wait(b->ctx[h], nullptr);
                return rc;
            }
            any = 1;
        }
        if (!any) break;
        for (int g = 0; g < G; ++g) {
            if (k[g] <= 0) continue;
            int rc = scft_iterate_wait(b->ctx[g], recs[g].data());
            if (rc != SCFT_OK) status = rc;
            ran[g] += k[g];
            const int Bg = (int)b->members[g].size();
            int all_done = 1;
            for (int s = 0; s < Bg; ++s) {
                const scft_iter_out &r = recs[g][(size_t)(k[g] - 1) * Bg + s];
                const int i = b->members[g][s];
                b->last[i] = r;
                b->iter[i] = r.iter;
                b->idle[i] = r.converged ? 1 : 0;
                if (!r.converged) all_done = 0;
            }
            if (all_done || status != SCFT_OK) live[g] = 0;
        }
        if (status != SCFT_OK) break;
    }
    if (res)
        for (int i = 0; i < b->n; ++i) {
            res[i].iterations = b->iter[i] - start[i];
            res[i].iter = b->iter[i];
            res[i].free_energy = b->last[i].free_energy;
            res[i].rms = b->last[i].rms;
            res[i].converged = b->last[i].converged;
            res[i].status = b->last[i].status;
        }
    return status;
}
