// mdg_serve.cpp -- continuous-batching server for independent simulation jobs.
//
// The server's slots (typed by kind, sized by particle capacity) live in one
// batch context per slot group (default: per particle kind), each with its
// own CUDA stream.  Jobs are
// submitted with their config, initial state and step count; pump() admits
// queued jobs into free slots while the estimated device footprint of the
// resident jobs stays within the HBM budget, advances every resident job with
// one multi-step launch per context -- all contexts' launches are queued
// before any is waited for, so the kinds' kernels run side by side on the GPU
// and one kind's latency-bound kernels fill the SMs the other leaves idle --
// (each job's step budget freezes it when done, so short jobs never run past
// their end), retires finished jobs (state downloaded, slot freed) and records
// submit / start / end times.  Job state stays on the device between pumps.
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <vector>

#include "../../include/mdg.h"

namespace {

using clk = std::chrono::steady_clock;

struct HostState {
    size_t n = 0;
    std::vector<uint32_t> tag, type;
    std::vector<double> pos, vel, force, mass, cutr, radius, inv_inertia, omega, torque, quat;
    std::vector<int32_t> image;
    bool dem = false;

    void take(const mdg_state_view& v, bool is_dem) {
        n = v.n;
        dem = is_dem;
        auto cp = [](auto* src, auto& dst, size_t k) {
            if (src) dst.assign(src, src + k);
            else dst.clear();
        };
        cp(v.tag, tag, n);
        cp(v.type, type, n);
        cp(v.pos, pos, 3 * n);
        cp(v.vel, vel, 3 * n);
        cp(v.force, force, 3 * n);
        cp(v.mass, mass, n);
        cp(v.cutoff_radius, cutr, n);
        cp(v.image, image, 3 * n);
        cp(v.radius, radius, n);
        cp(v.inv_inertia, inv_inertia, n);
        cp(v.omega, omega, 3 * n);
        cp(v.torque, torque, 3 * n);
        cp(v.quat, quat, 4 * n);
    }
    void alloc(size_t k, bool is_dem) {
        n = k;
        dem = is_dem;
        tag.assign(n, 0);
        type.assign(n, 0);
        pos.assign(3 * n, 0.0);
        vel.assign(3 * n, 0.0);
        force.assign(3 * n, 0.0);
        mass.assign(n, 0.0);
        cutr.assign(n, 0.0);
        image.assign(3 * n, 0);
        if (dem) {
            radius.assign(n, 0.0);
            inv_inertia.assign(n, 0.0);
            omega.assign(3 * n, 0.0);
            torque.assign(3 * n, 0.0);
            quat.assign(4 * n, 0.0);
        }
    }
    mdg_state_view view() {
        mdg_state_view v{};
        v.n = n;
        auto p = [](auto& vec) { return vec.empty() ? nullptr : vec.data(); };
        v.tag = p(tag);
        v.type = p(type);
        v.pos = p(pos);
        v.vel = p(vel);
        v.force = p(force);
        v.mass = p(mass);
        v.cutoff_radius = p(cutr);
        v.image = p(image);
        v.radius = p(radius);
        v.inv_inertia = p(inv_inertia);
        v.omega = p(omega);
        v.torque = p(torque);
        v.quat = p(quat);
        return v;
    }
};

struct Job {
    int64_t id = 0;
    mdg_config cfg{};
    // owned copies of the arrays cfg points at (the caller's may be gone by admission)
    std::vector<mdg_material> mats;
    std::vector<mdg_wall> walls;
    std::vector<mdg_lj_pair> ljp;
    HostState state;
    int64_t steps = 0;
    int64_t left = 0;  // steps still to run while resident
    size_t bytes = 0;
    int slot = -1;
    int status = MDG_OK;
    double t_submit = 0, t_start = -1, t_end = -1;
};

// Device footprint of a job, used for admission: the per-particle state and
// scratch arrays, the neighbour rows and (DEM) the two contact-history buffers.
size_t job_bytes(const mdg_config& c, size_t n) {
    const size_t per = 32 * 12 + 8 * 4 + 16 * 4 + 64;  // SoA rows, gather scratch, two-float copies
    const size_t rows = (c.kind == MDG_KIND_LJ ? 128 : 48) * 4;
    const size_t hist = c.kind == MDG_KIND_DEM ? 3 * 24 * 60 : 0;
    return n * (per + rows + hist);
}

}  // namespace

struct mdg_server {
    std::vector<mdg_ctx*> ctxs;    // one batch context per particle kind present
    std::vector<int> slot_ctx;     // slot -> its context
    std::vector<int> slot_sys;     // slot -> its system index in that context
    int nslots = 0;
    std::vector<int> slot_kind;
    std::vector<size_t> slot_cap;
    std::vector<int64_t> slot_job;  // -1 free
    size_t budget = 0, used = 0;
    int64_t next_id = 1;
    std::deque<int64_t> pending;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    std::vector<int64_t> finished;  // not yet polled
    double particle_steps = 0;  // work done by all pumps
    double admit_s = 0, step_s = 0, retire_s = 0;
    int64_t pumps = 0, retired = 0;
    clk::time_point t0 = clk::now();
    double now() const { return std::chrono::duration<double>(clk::now() - t0).count(); }
};

extern "C" {

int mdg_server_create_grouped(const mdg_config* slot_cfgs, const size_t* slot_capacity, const int* slot_group,
                              int nslots, size_t hbm_budget, mdg_server** out) {
    if (!slot_cfgs || !slot_capacity || !slot_group || nslots < 1 || !out) return MDG_ERR_ARG;
    *out = nullptr;
    for (int k = 0; k < nslots; k++) {
        if (slot_cfgs[k].kind != MDG_KIND_DEM && slot_cfgs[k].kind != MDG_KIND_LJ) return MDG_ERR_CONFIG;
        for (int q = 0; q < k; q++)  // a group holds one kind
            if (slot_group[q] == slot_group[k] && slot_cfgs[q].kind != slot_cfgs[k].kind) return MDG_ERR_CONFIG;
    }
    auto* s = new (std::nothrow) mdg_server();
    if (!s) return MDG_ERR_OOM;
    s->nslots = nslots;
    s->slot_ctx.assign(nslots, -1);
    s->slot_sys.assign(nslots, -1);
    // the slots of each group, in slot order, make one batch context; groups
    // in order of their first slot
    for (int k0 = 0; k0 < nslots; k0++) {
        if (s->slot_ctx[k0] >= 0) continue;
        std::vector<mdg_config> cfgs;
        std::vector<size_t> caps;
        std::vector<int> ids;
        for (int k = k0; k < nslots; k++)
            if (slot_group[k] == slot_group[k0]) {
                cfgs.push_back(slot_cfgs[k]);
                caps.push_back(slot_capacity[k]);
                ids.push_back(k);
            }
        mdg_ctx* ctx = nullptr;
        const int r = mdg_batch_create(cfgs.data(), caps.data(), (int)cfgs.size(), &ctx);
        if (r) {
            for (mdg_ctx* c : s->ctxs) mdg_destroy(c);
            delete s;
            return r;
        }
        for (size_t q = 0; q < ids.size(); q++) {
            s->slot_ctx[ids[q]] = (int)s->ctxs.size();
            s->slot_sys[ids[q]] = (int)q;
            mdg_set_remaining(ctx, (int)q, 0);
        }
        s->ctxs.push_back(ctx);
    }
    for (int k = 0; k < nslots; k++) {
        s->slot_kind.push_back(slot_cfgs[k].kind);
        s->slot_cap.push_back(slot_capacity[k]);
        s->slot_job.push_back(-1);
    }
    s->budget = hbm_budget;
    *out = s;
    return MDG_OK;
}

int mdg_server_create(const mdg_config* slot_cfgs, const size_t* slot_capacity, int nslots, size_t hbm_budget,
                      mdg_server** out) {
    if (!slot_cfgs || nslots < 1) return MDG_ERR_ARG;
    std::vector<int> group(nslots);
    for (int k = 0; k < nslots; k++) group[k] = slot_cfgs[k].kind;  // one context per particle kind
    return mdg_server_create_grouped(slot_cfgs, slot_capacity, group.data(), nslots, hbm_budget, out);
}

void mdg_server_destroy(mdg_server* s) {
    if (!s) return;
    for (mdg_ctx* c : s->ctxs) mdg_destroy(c);
    delete s;
}

int mdg_server_submit(mdg_server* s, const mdg_config* cfg, const mdg_state_view* st, int64_t steps, int64_t* id) {
    if (!s || !cfg || !st || !id || steps < 0 || st->n < 1) return MDG_ERR_ARG;
    bool fits = false;
    for (int k = 0; k < s->nslots; k++)
        if (s->slot_kind[k] == cfg->kind && s->slot_cap[k] >= st->n) fits = true;
    if (!fits) return MDG_ERR_BUDGET;  // no slot could ever hold it
    auto j = std::make_unique<Job>();
    j->id = s->next_id++;
    j->cfg = *cfg;
    if (cfg->kind == MDG_KIND_DEM && cfg->materials && cfg->n_materials > 0) {
        j->mats.assign(cfg->materials, cfg->materials + cfg->n_materials);
        j->cfg.materials = j->mats.data();
    }
    if (cfg->walls && cfg->n_walls > 0 && cfg->n_walls <= MDG_MAX_WALLS) {
        j->walls.assign(cfg->walls, cfg->walls + cfg->n_walls);
        j->cfg.walls = j->walls.data();
    }
    if (cfg->kind == MDG_KIND_LJ && cfg->lj_pairs && cfg->n_lj_types > 1) {
        j->ljp.assign(cfg->lj_pairs, cfg->lj_pairs + (size_t)cfg->n_lj_types * cfg->n_lj_types);
        j->cfg.lj_pairs = j->ljp.data();
    }
    j->state.take(*st, cfg->kind == MDG_KIND_DEM);
    j->steps = steps;
    j->bytes = job_bytes(*cfg, st->n);
    if (j->bytes > s->budget) return MDG_ERR_BUDGET;
    j->t_submit = s->now();
    *id = j->id;
    s->pending.push_back(j->id);
    s->jobs[j->id] = std::move(j);
    return MDG_OK;
}

// Admit, advance up to max_steps, retire.  active/pending report the counts
// after the call.
int mdg_server_pump(mdg_server* s, int64_t max_steps, int* active, int* pending) {
    if (!s || max_steps < 0) return MDG_ERR_ARG;
    const double ta = s->now();
    // admission: FIFO, skipping jobs that do not fit yet (no head-of-line blocking)
    for (auto it = s->pending.begin(); it != s->pending.end();) {
        Job* j = s->jobs[*it].get();
        int slot = -1;
        size_t best = (size_t)-1;
        for (int k = 0; k < s->nslots; k++)
            if (s->slot_job[k] < 0 && s->slot_kind[k] == j->cfg.kind && s->slot_cap[k] >= j->state.n &&
                s->slot_cap[k] < best) {
                best = s->slot_cap[k];
                slot = k;
            }
        if (slot < 0 || s->used + j->bytes > s->budget) {
            ++it;
            continue;
        }
        mdg_ctx* ctx = s->ctxs[s->slot_ctx[slot]];
        const int sys = s->slot_sys[slot];
        int r = mdg_configure_system(ctx, sys, &j->cfg);
        mdg_state_view v = j->state.view();
        if (!r) r = mdg_upload_state(ctx, sys, &v);
        if (!r) r = mdg_set_remaining(ctx, sys, j->steps);
        if (r) {  // the job cannot run: finish it with its error
            j->status = r;
            j->t_start = j->t_end = s->now();
            s->finished.push_back(j->id);
            it = s->pending.erase(it);
            continue;
        }
        j->slot = slot;
        j->left = j->steps;
        j->t_start = s->now();
        s->slot_job[slot] = j->id;
        s->used += j->bytes;
        it = s->pending.erase(it);
    }
    const int nctx = (int)s->ctxs.size();
    int nactive = 0;
    std::vector<int64_t> most(nctx, 0);
    for (int k = 0; k < s->nslots; k++)
        if (s->slot_job[k] >= 0) {
            // a resident job's budget is exactly its steps left: the host
            // tracks it, the device counts it down
            const int64_t left = s->jobs[s->slot_job[k]]->left;
            int64_t& m = most[s->slot_ctx[k]];
            m = left > m ? left : m;
            nactive++;
        }
    const double tb = s->now();
    s->admit_s += tb - ta;
    int rstep = MDG_OK;
    // every context's launch is queued before any is waited for
    std::vector<int64_t> adv(nctx, 0);
    bool stepped = false;
    for (int g = 0; g < nctx; g++) {
        adv[g] = most[g] < max_steps ? most[g] : max_steps;
        if (adv[g] <= 0) continue;
        const int r = mdg_step_async(s->ctxs[g], adv[g]);
        if (r && rstep == MDG_OK) rstep = r;
        if (r) adv[g] = 0;
        stepped = true;
    }
    for (int g = 0; g < nctx; g++) {
        if (adv[g] <= 0) continue;
        const int r = mdg_step_wait(s->ctxs[g]);
        if (r && rstep == MDG_OK) rstep = r;
    }
    if (stepped) {
        for (int k = 0; k < s->nslots; k++)
            if (s->slot_job[k] >= 0) {
                const Job* j = s->jobs[s->slot_job[k]].get();
                const int64_t a = adv[s->slot_ctx[k]];
                s->particle_steps += (double)j->state.n * (double)(j->left < a ? j->left : a);
            }
        s->pumps++;
    }
    const double tc = s->now();
    s->step_s += tc - tb;
    // retirement: one read of every context's budgets and statuses
    std::vector<std::vector<int64_t>> left(nctx);
    std::vector<std::vector<int32_t>> stw(nctx);
    if (nactive)
        for (int g = 0; g < nctx; g++) {
            const int ns = mdg_num_systems(s->ctxs[g]);
            left[g].assign(ns, 0);
            stw[g].assign(ns, 0);
            const int r = mdg_get_progress(s->ctxs[g], left[g].data(), stw[g].data(), nullptr);
            if (r) return r;
        }
    for (int k = 0; k < s->nslots; k++) {
        if (s->slot_job[k] < 0) continue;
        const int g = s->slot_ctx[k], sys = s->slot_sys[k];
        s->jobs[s->slot_job[k]]->left = left[g][sys];
        const bool failed = stw[g][sys] != 0;
        if (left[g][sys] != 0 && !failed) continue;
        Job* j = s->jobs[s->slot_job[k]].get();
        j->state.alloc(j->state.n, j->cfg.kind == MDG_KIND_DEM);
        mdg_state_view v = j->state.view();
        const int rd = mdg_download_state(s->ctxs[g], sys, &v);
        j->status = failed ? (rstep != MDG_OK ? rstep : MDG_ERR_STATE) : rd;
        j->t_end = s->now();
        s->finished.push_back(j->id);
        s->retired++;
        s->used -= j->bytes;
        s->slot_job[k] = -1;
        mdg_set_remaining(s->ctxs[g], sys, 0);
        nactive--;
    }
    s->retire_s += s->now() - tc;
    if (active) *active = nactive;
    if (pending) *pending = (int)s->pending.size();
    return (rstep == MDG_OK || rstep == MDG_ERR_OVERLAP_LIMIT || rstep == MDG_ERR_NAN ||
            rstep == MDG_ERR_LIST_OVERFLOW) ? MDG_OK : rstep;
}

int mdg_server_stats(mdg_server* s, mdg_server_stats_t* out) {
    if (!s || !out) return MDG_ERR_ARG;
    out->particle_steps = s->particle_steps;
    out->pumps = s->pumps;
    out->retired = s->retired;
    int resident = 0;
    for (int k = 0; k < s->nslots; k++) resident += s->slot_job[k] >= 0;
    out->resident = resident;
    out->pending = (int)s->pending.size();
    out->hbm_used = s->used;
    out->time_s = s->now();
    out->admit_s = s->admit_s;
    out->step_s = s->step_s;
    out->retire_s = s->retire_s;
    out->launches = 0;
    for (mdg_ctx* c : s->ctxs) out->launches += mdg_kernel_launches(c);
    out->contexts = (int32_t)s->ctxs.size();
    return MDG_OK;
}

int mdg_server_resident(mdg_server* s, mdg_job_info* out, int cap, int* n) {
    if (!s || !n || (cap > 0 && !out)) return MDG_ERR_ARG;
    int m = 0;
    for (int k = 0; k < s->nslots; k++) {
        if (s->slot_job[k] < 0) continue;
        if (m < cap) {
            const Job* j = s->jobs[s->slot_job[k]].get();
            mdg_job_info& o = out[m];
            o.id = j->id;
            o.status = j->status;
            o.slot = k;
            o.steps = j->steps - j->left;  // steps done so far
            o.n = (int64_t)j->state.n;
            o.submit_s = j->t_submit;
            o.start_s = j->t_start;
            o.end_s = -1.0;
        }
        m++;
    }
    *n = m;
    return MDG_OK;
}

int mdg_server_poll(mdg_server* s, mdg_job_info* out, int cap, int* n) {
    if (!s || !n || (cap > 0 && !out)) return MDG_ERR_ARG;
    int m = 0;
    while (m < cap && !s->finished.empty()) {
        Job* j = s->jobs[s->finished.front()].get();
        s->finished.erase(s->finished.begin());
        mdg_job_info& o = out[m++];
        o.id = j->id;
        o.status = j->status;
        o.slot = j->slot;
        o.steps = j->steps;
        o.n = (int64_t)j->state.n;
        o.submit_s = j->t_submit;
        o.start_s = j->t_start;
        o.end_s = j->t_end;
    }
    *n = m;
    return MDG_OK;
}

int mdg_server_fetch(mdg_server* s, int64_t id, mdg_state_view* out) {
    if (!s || !out) return MDG_ERR_ARG;
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return MDG_ERR_ARG;
    Job* j = it->second.get();
    if (j->t_end < 0) return MDG_ERR_STATE;
    if (out->n < j->state.n) return MDG_ERR_ARG;
    const size_t n = j->state.n;
    HostState& h = j->state;
    auto cp = [](auto* dst, const auto& src) {
        if (dst && !src.empty()) std::memcpy(dst, src.data(), src.size() * sizeof(src[0]));
    };
    out->n = n;
    cp(out->tag, h.tag);
    cp(out->type, h.type);
    cp(out->pos, h.pos);
    cp(out->vel, h.vel);
    cp(out->force, h.force);
    cp(out->mass, h.mass);
    cp(out->cutoff_radius, h.cutr);
    cp(out->image, h.image);
    cp(out->radius, h.radius);
    cp(out->inv_inertia, h.inv_inertia);
    cp(out->omega, h.omega);
    cp(out->torque, h.torque);
    cp(out->quat, h.quat);
    s->jobs.erase(it);
    return MDG_OK;
}

int mdg_server_context(mdg_server* s, mdg_ctx** ctx) {
    if (!s || !ctx) return MDG_ERR_ARG;
    *ctx = s->ctxs[s->slot_ctx[0]];
    return MDG_OK;
}

int mdg_server_slot_context(mdg_server* s, int slot, mdg_ctx** ctx, int* sys) {
    if (!s || !ctx || !sys || slot < 0 || slot >= s->nslots) return MDG_ERR_ARG;
    *ctx = s->ctxs[s->slot_ctx[slot]];
    *sys = s->slot_sys[slot];
    return MDG_OK;
}

}  // extern "C"
