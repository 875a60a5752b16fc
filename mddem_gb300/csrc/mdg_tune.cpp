// mdg_tune.cpp -- autotuner for the batched hot path (host, on the C ABI).
//
// Knobs (all physics-neutral): the LJ force kernel's lanes per particle row,
// and per particle kind the skin fraction (rebuild cadence) and the bin size
// (multiple of the list cutoff).  Each trial re-uploads the saved initial
// state of every system under the trial's configs and times graph-launched
// steps; coordinate descent keeps the cheapest value of one knob at a time.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/mdg.h"

namespace {

struct Saved {
    bool dem = false;
    size_t n = 0;
    std::vector<uint32_t> tag, type;
    std::vector<double> pos, vel, force, mass, cutr, radius, inv_inertia, omega, torque, quat;
    std::vector<int32_t> image;
    std::vector<uint32_t> hkeys;
    std::vector<double> hvals;
    int64_t remaining = -1;
    mdg_config cfg{};
    std::vector<mdg_material> mats;
    double max_r = 0.0;

    mdg_state_view view() {
        mdg_state_view v{};
        v.n = n;
        auto p = [](auto& x) { return x.empty() ? nullptr : x.data(); };
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

int save_system(mdg_ctx* c, int s, Saved& sv) {
    mdg_thermo_t t{};
    int r = mdg_thermo(c, s, &t);
    if (r) return r;
    if (t.step != 0) return MDG_ERR_STATE;  // tune before the first step
    r = mdg_get_config(c, s, &sv.cfg);
    if (r) return r;
    sv.mats.assign(sv.cfg.materials, sv.cfg.materials + (sv.cfg.materials ? sv.cfg.n_materials : 0));
    sv.cfg.materials = sv.mats.empty() ? nullptr : sv.mats.data();
    sv.dem = sv.cfg.kind == MDG_KIND_DEM;
    sv.n = (size_t)t.n;
    const size_t n = sv.n;
    sv.tag.resize(n);
    sv.type.resize(n);
    sv.pos.resize(3 * n);
    sv.vel.resize(3 * n);
    sv.force.resize(3 * n);
    sv.mass.resize(n);
    sv.cutr.resize(n);
    sv.image.resize(3 * n);
    if (sv.dem) {
        sv.radius.resize(n);
        sv.inv_inertia.resize(n);
        sv.omega.resize(3 * n);
        sv.torque.resize(3 * n);
        sv.quat.resize(4 * n);
    }
    mdg_state_view v = sv.view();
    r = mdg_download_state(c, s, &v);
    if (r) return r;
    for (double x : sv.cutr) sv.max_r = std::max(sv.max_r, x);
    if (sv.dem) {
        size_t m = 0;
        r = mdg_get_history(c, s, nullptr, nullptr, 0, &m);
        if (r) return r;
        sv.hkeys.resize(2 * m);
        sv.hvals.resize(7 * m);
        if (m) r = mdg_get_history(c, s, sv.hkeys.data(), sv.hvals.data(), m, &m);
        if (r) return r;
    }
    return mdg_get_remaining(c, s, &sv.remaining);
}

// The trial's knobs per kind: skin fraction and bin factor (0 = as saved).
struct Knobs {
    double skin[2] = {0, 0};
    double binf[2] = {0, 0};
};

int kind_index(const Saved& sv) { return sv.dem ? 0 : 1; }

mdg_config trial_config(const Saved& sv, const Knobs& k) {
    mdg_config cfg = sv.cfg;
    const int q = kind_index(sv);
    if (k.skin[q] > 0.0) cfg.skin_fraction = k.skin[q];
    if (k.binf[q] > 0.0) cfg.bin_size = k.binf[q] * 2.0 * sv.max_r * cfg.skin_fraction;
    return cfg;
}

int load_all(mdg_ctx* c, std::vector<Saved>& sys, const std::vector<int>& ids, const Knobs& k) {
    for (size_t q = 0; q < ids.size(); q++) {
        Saved& sv = sys[q];
        const int s = ids[q];
        mdg_config cfg = trial_config(sv, k);
        int r = mdg_configure_system(c, s, &cfg);
        mdg_state_view v = sv.view();
        if (!r) r = mdg_upload_state(c, s, &v);
        if (!r && !sv.hkeys.empty()) r = mdg_set_history(c, s, sv.hvals.size() / 7, sv.hkeys.data(), sv.hvals.data());
        if (!r && sv.remaining != -1) r = mdg_set_remaining(c, s, sv.remaining);
        if (r) return r;
    }
    return MDG_OK;
}

// Modelled ms per step of the current configuration; < 0 on failure.
double trial(mdg_ctx* c, std::vector<Saved>& sys, const std::vector<int>& ids, const Knobs& k, int steps) {
    if (load_all(c, sys, ids, k)) return -1.0;
    std::vector<mdg_step_timing> t((size_t)steps * 8 + 1);
    // step 0 rebuilds every system from scratch: its excess is the full
    // rebuild cost; then warm-up
    if (mdg_timed_steps(c, 1, 0, t.data())) return -1.0;
    const double first = t[0].step_ms;
    if (mdg_timed_steps(c, 3, 0, t.data())) return -1.0;
    int done = 0, rebuilds = 0;
    double sum = 0.0, quiet = 0.0;
    int nquiet = 0;
    while (done < steps * 8) {
        const int m = steps;
        if (mdg_timed_steps(c, m, 0, t.data())) return -1.0;
        for (int q = 0; q < m; q++) {
            sum += t[q].step_ms;
            if (t[q].rebuilt) rebuilds++;
            else {
                quiet += t[q].step_ms;
                nquiet++;
            }
        }
        done += m;
        if (done >= steps && rebuilds >= 2) break;
    }
    double cost = sum / done;
    if (rebuilds == 0 && nquiet > 0) cost = quiet / nquiet + std::max(0.0, first - quiet / nquiet) / done;
    int32_t st = 0;
    for (int s : ids) {
        mdg_get_status(c, s, &st);
        if (st) return -1.0;  // e.g. list overflow under this trial: reject it
    }
    return cost;
}

}  // namespace

extern "C" int mdg_autotune(mdg_ctx* c, const mdg_tune_opts* o, mdg_tune_result* out) {
    if (!c || !out) return MDG_ERR_ARG;
    mdg_tune_opts opts = o ? *o : mdg_tune_opts{0, 1, 1, 1};
    const int steps = opts.steps > 0 ? opts.steps : 40;
    std::memset(out, 0, sizeof(*out));
    std::vector<Saved> sys;
    std::vector<int> ids;
    bool has[2] = {false, false};
    for (int s = 0; s < mdg_num_systems(c); s++) {
        Saved sv;
        mdg_thermo_t t{};
        if (mdg_thermo(c, s, &t) == MDG_ERR_STATE) continue;  // not uploaded
        int r = save_system(c, s, sv);
        if (r) return r;
        has[kind_index(sv)] = true;
        sys.push_back(std::move(sv));
        ids.push_back(s);
    }
    if (ids.empty()) return MDG_ERR_STATE;
    Knobs best;
    int tpp = mdg_get_threads_per_particle(c);
    double best_ms = trial(c, sys, ids, best, steps);
    if (best_ms < 0) return MDG_ERR_STATE;
    out->ms_before = best_ms;
    int trials = 1;
    if (opts.tune_tpp && has[1]) {
        for (int cand : {1, 2, 4, 8}) {
            if (cand == tpp) continue;
            mdg_set_threads_per_particle(c, cand);
            const double ms = trial(c, sys, ids, best, steps);
            trials++;
            if (ms >= 0 && ms < best_ms) {
                best_ms = ms;
                tpp = cand;
            }
        }
        mdg_set_threads_per_particle(c, tpp);
    }
    static const double skins[2][5] = {{1.05, 1.1, 1.2, 1.35, 1.5}, {1.08, 1.12, 1.2, 1.3, 1.4}};
    static const double bins[4] = {1.0, 1.3, 1.7, 2.2};
    for (int q = 0; q < 2; q++) {
        if (!has[q]) continue;
        if (opts.tune_skin) {
            for (double sk : skins[q]) {
                Knobs k = best;
                k.skin[q] = sk;
                const double ms = trial(c, sys, ids, k, steps);
                trials++;
                if (ms >= 0 && ms < best_ms) {
                    best_ms = ms;
                    best = k;
                }
            }
        }
        if (opts.tune_bin) {
            for (double bf : bins) {
                Knobs k = best;
                k.binf[q] = bf;
                const double ms = trial(c, sys, ids, k, steps);
                trials++;
                if (ms >= 0 && ms < best_ms) {
                    best_ms = ms;
                    best = k;
                }
            }
        }
    }
    // leave the systems as uploaded, under the chosen parameters
    const int r = load_all(c, sys, ids, best);
    if (r) return r;
    out->tpp = tpp;
    for (int q = 0; q < 2; q++) {
        if (!has[q]) continue;
        const Saved* any = nullptr;
        for (const Saved& sv : sys)
            if (kind_index(sv) == q) any = &sv;
        const mdg_config cfg = trial_config(*any, best);
        out->skin_fraction[q] = cfg.skin_fraction;
        // the grid's bins are at least the list cutoff (compute_bin_grid)
        out->bin_factor[q] = std::max(1.0, cfg.bin_size / (2.0 * any->max_r * cfg.skin_fraction));
    }
    out->ms_after = best_ms;
    out->trials = trials;
    return MDG_OK;
}
