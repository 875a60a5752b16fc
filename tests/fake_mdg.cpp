// fake_mdg.cpp -- test infrastructure: a CPU stand-in for libmddem_gb300.so
// with the entry points the C++ host calls, so the host's run path (create,
// upload, steps between outputs, thermo, download, history, restart files,
// resume) runs without a GPU.  Particles fly freely (x += v dt per step) and
// keep the force and torque they were uploaded with; every call checks its
// arguments against the uploaded state and logs itself to stderr.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../include/mdg.h"

struct mdg_ctx {
    mdg_config cfg;
    size_t cap = 0, n = 0;
    bool dem = false, uploaded = false;
    long long step = 0;
    std::vector<uint32_t> tag, type;
    std::vector<double> pos, vel, force, torque, mass, cutr, radius, inv_inertia, omega, quat;
    bool history_set = false;
    std::vector<uint32_t> hkeys;
    std::vector<double> hvals;
};

extern "C" {

const char* mdg_status_string(int s) { return s == MDG_OK ? "ok" : "fake error"; }

int mdg_create(const mdg_config* cfg, size_t capacity, mdg_ctx** out) {
    if (!cfg || !out || cfg->dt <= 0.0) return MDG_ERR_CONFIG;
    mdg_ctx* c = new mdg_ctx();
    c->cfg = *cfg;
    c->cap = capacity;
    c->dem = cfg->kind == MDG_KIND_DEM;
    *out = c;
    std::fprintf(stderr, "fake: create kind=%d capacity=%zu materials=%d walls=%d lj_types=%d\n", cfg->kind,
                 capacity, cfg->n_materials, cfg->n_walls, cfg->n_lj_types);
    if (cfg->n_lj_types > 1) {
        if (!cfg->lj_pairs) return MDG_ERR_CONFIG;
        for (int k = 0; k < cfg->n_lj_types * cfg->n_lj_types; k++)
            std::fprintf(stderr, "fake: lj_pair %d %.17g %.17g %.17g\n", k, cfg->lj_pairs[k].epsilon,
                         cfg->lj_pairs[k].sigma, cfg->lj_pairs[k].cutoff);
    }
    return MDG_OK;
}

void mdg_destroy(mdg_ctx* c) { delete c; }

int mdg_upload_state(mdg_ctx* c, int sys, const mdg_state_view* v) {
    if (!c || sys != 0 || !v || v->n > c->cap || !v->tag || !v->pos || !v->vel || !v->mass || !v->cutoff_radius)
        return MDG_ERR_ARG;
    if (c->dem && (!v->radius || !v->inv_inertia || !v->omega || !v->quat)) return MDG_ERR_ARG;
    const size_t n = v->n;
    if (c->cfg.n_lj_types > 1)
        for (size_t i = 0; i < n; i++)
            if (!v->type || v->type[i] >= (uint32_t)c->cfg.n_lj_types) return MDG_ERR_ARG;
    c->n = n;
    c->tag.assign(v->tag, v->tag + n);
    c->type.assign(v->type, v->type + n);
    c->pos.assign(v->pos, v->pos + 3 * n);
    c->vel.assign(v->vel, v->vel + 3 * n);
    c->force.assign(3 * n, 0.0);
    if (v->force) c->force.assign(v->force, v->force + 3 * n);
    c->torque.assign(3 * n, 0.0);
    if (c->dem && v->torque) c->torque.assign(v->torque, v->torque + 3 * n);
    c->mass.assign(v->mass, v->mass + n);
    c->cutr.assign(v->cutoff_radius, v->cutoff_radius + n);
    if (c->dem) {
        c->radius.assign(v->radius, v->radius + n);
        c->inv_inertia.assign(v->inv_inertia, v->inv_inertia + n);
        c->omega.assign(v->omega, v->omega + 3 * n);
        c->quat.assign(v->quat, v->quat + 4 * n);
    }
    c->uploaded = true;
    std::fprintf(stderr, "fake: upload n=%zu force=%d torque=%d\n", n, v->force != nullptr,
                 c->dem && v->torque != nullptr);
    return MDG_OK;
}

int mdg_step(mdg_ctx* c, int64_t k) {
    if (!c || !c->uploaded || k < 0) return MDG_ERR_STATE;
    for (size_t i = 0; i < 3 * c->n; i++) c->pos[i] += c->vel[i] * c->cfg.dt * (double)k;
    c->step += k;
    std::fprintf(stderr, "fake: step %lld\n", (long long)k);
    return MDG_OK;
}

int mdg_thermo(mdg_ctx* c, int sys, mdg_thermo_t* t) {
    if (!c || sys != 0 || !t || !c->uploaded) return MDG_ERR_ARG;
    std::memset(t, 0, sizeof(*t));
    double m = 0, ke = 0;
    for (size_t i = 0; i < c->n; i++) {
        const double* v = &c->vel[3 * i];
        ke += 0.5 * c->mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        m += c->mass[i];
    }
    t->ke = ke;
    t->temp = c->n > 1 ? 2.0 * ke / (3.0 * (double)c->n - 3.0) : 0.0;
    t->granular_temp = m > 0 ? 2.0 * ke / (3.0 * m) : 0.0;
    t->step = c->step;
    t->n = (int64_t)c->n;
    return MDG_OK;
}

int mdg_download_state(mdg_ctx* c, int sys, mdg_state_view* v) {
    if (!c || sys != 0 || !v || v->n != c->n || !v->tag || !v->pos || !v->vel) return MDG_ERR_ARG;
    const size_t n = c->n;
    std::memcpy(v->tag, c->tag.data(), n * sizeof(uint32_t));
    if (v->type) std::memcpy(v->type, c->type.data(), n * sizeof(uint32_t));
    std::memcpy(v->pos, c->pos.data(), 3 * n * sizeof(double));
    std::memcpy(v->vel, c->vel.data(), 3 * n * sizeof(double));
    if (v->force) std::memcpy(v->force, c->force.data(), 3 * n * sizeof(double));
    if (v->mass) std::memcpy(v->mass, c->mass.data(), n * sizeof(double));
    if (v->cutoff_radius) std::memcpy(v->cutoff_radius, c->cutr.data(), n * sizeof(double));
    if (v->image) std::memset(v->image, 0, 3 * n * sizeof(int32_t));
    if (c->dem) {
        if (!v->radius || !v->inv_inertia || !v->omega || !v->quat) return MDG_ERR_ARG;
        std::memcpy(v->radius, c->radius.data(), n * sizeof(double));
        std::memcpy(v->inv_inertia, c->inv_inertia.data(), n * sizeof(double));
        std::memcpy(v->omega, c->omega.data(), 3 * n * sizeof(double));
        std::memcpy(v->quat, c->quat.data(), 4 * n * sizeof(double));
        if (v->torque) std::memcpy(v->torque, c->torque.data(), 3 * n * sizeof(double));
    }
    return MDG_OK;
}

int mdg_set_history(mdg_ctx* c, int sys, size_t n, const uint32_t* keys, const double* vals) {
    if (!c || sys != 0 || !c->dem || !c->uploaded || (n && (!keys || !vals))) return MDG_ERR_ARG;
    c->hkeys.assign(keys, keys + 2 * n);
    c->hvals.assign(vals, vals + 7 * n);
    c->history_set = true;
    std::fprintf(stderr, "fake: set_history n=%zu\n", n);
    return MDG_OK;
}

// the history that was set, else one synthetic contact (tag 0 with tag 1)
// when the system has two particles
int mdg_get_history(mdg_ctx* c, int sys, uint32_t* keys, double* vals, size_t cap, size_t* n) {
    if (!c || sys != 0 || !n) return MDG_ERR_ARG;
    if (c->history_set) {
        const size_t have = c->hkeys.size() / 2;
        if (cap >= have && have) {
            std::memcpy(keys, c->hkeys.data(), 2 * have * sizeof(uint32_t));
            std::memcpy(vals, c->hvals.data(), 7 * have * sizeof(double));
        }
        *n = have;
        return MDG_OK;
    }
    const size_t have = (c->dem && c->n >= 2) ? 1 : 0;
    if (cap >= have && have) {
        keys[0] = 0;
        keys[1] = 1;
        for (int q = 0; q < 7; q++) vals[q] = 0.5 * (q + 1);
    }
    *n = have;
    return MDG_OK;
}

int mdg_rdf(mdg_ctx* c, int sys, double, int nbins, uint64_t* counts) {
    if (!c || sys != 0 || nbins <= 0 || !counts) return MDG_ERR_ARG;
    for (int k = 0; k < nbins; k++) counts[k] = 1;
    return MDG_OK;
}
int mdg_msd_reset(mdg_ctx* c, int sys) { return (c && sys == 0) ? MDG_OK : MDG_ERR_ARG; }
int mdg_msd(mdg_ctx* c, int sys, double* msd) {
    if (!c || sys != 0 || !msd) return MDG_ERR_ARG;
    *msd = (double)c->step;
    return MDG_OK;
}

// spheres on a grid inside the box (no rejection): enough for host tests
int mdg_rsa_spheres(size_t n, const double lo[3], const double hi[3], double rmin, double rmax, double, int inset,
                    uint64_t, uint64_t, double* pos, double* rad, size_t* placed) {
    const int side = (int)std::ceil(std::cbrt((double)n));
    for (size_t i = 0; i < n; i++) {
        const size_t g[3] = {i % side, (i / side) % side, i / ((size_t)side * side)};
        for (int d = 0; d < 3; d++) {
            const double a = lo[d] + (inset ? rmax : 0.0), b = hi[d] - (inset ? rmax : 0.0);
            pos[3 * i + d] = a + (b - a) * (g[d] + 0.5) / side;
        }
        rad[i] = 0.5 * (rmin + rmax);
    }
    if (placed) *placed = n;
    return MDG_OK;
}

// The device generators are not faked: a config that asks for them needs a GPU.
int mdg_generate_fcc(mdg_ctx*, int, const mdg_fcc_spec*, size_t*) { return MDG_ERR_NODEVICE; }
int mdg_generate_gas(mdg_ctx*, int, const mdg_gas_spec*, size_t*) { return MDG_ERR_NODEVICE; }

}  // extern "C"
