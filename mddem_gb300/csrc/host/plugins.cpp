// plugins.cpp -- the granular and LJ plugin groups, walls, Langevin,
// measurements, and the JSON summary of a resolved configuration.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <limits>
#include <random>
#include <sstream>
#include <unordered_map>

#include "plugins.hpp"
#include "restart.hpp"

namespace mdg_host {
namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// granular group
// ---------------------------------------------------------------------------

// DemAtomPlugin: [[dem.materials]] (crates/dem_atom/src/lib.rs:78-158).
struct DemAtomPlugin : Plugin {
    std::string name() const override { return "DemAtomPlugin"; }
    std::vector<std::string> provides() const override { return {"dem_particles"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* dem = section(a, "dem");
            std::vector<const toml::Table*> ms;
            if (dem) ms = table_array(*dem, "materials");
            if (ms.empty()) throw ConfigError("[[dem.materials]] requires at least one material");
            for (const toml::Table* m : ms) {
                check_keys("dem.materials", *m,
                           {"name", "youngs_mod", "poisson_ratio", "restitution", "friction", "rolling_friction",
                            "twisting_friction", "cohesion_energy", "surface_energy", "kn", "kt", "rolling_stiffness",
                            "rolling_damping", "twisting_stiffness", "twisting_damping"});
                mdg_material x{};
                x.youngs_mod = num(m, "youngs_mod", 8.7e9);
                x.poisson_ratio = num(m, "poisson_ratio", 0.3);
                x.restitution = num(m, "restitution", 0.95);
                x.friction = num(m, "friction", 0.4);
                x.rolling_friction = num(m, "rolling_friction", 0.0);
                x.twisting_friction = num(m, "twisting_friction", 0.0);
                x.cohesion_energy = num(m, "cohesion_energy", 0.0);
                x.surface_energy = num(m, "surface_energy", 0.0);
                x.kn = num(m, "kn", 0.0);
                x.kt = num(m, "kt", 0.0);
                x.rolling_stiffness = num(m, "rolling_stiffness", 0.0);
                x.rolling_damping = num(m, "rolling_damping", 0.0);
                x.twisting_stiffness = num(m, "twisting_stiffness", 0.0);
                x.twisting_damping = num(m, "twisting_damping", 0.0);
                a.materials.push_back(x);
                a.material_names.push_back(text(m, "name", "glass"));
            }
        });
    }
};

// HertzMindlinContactPlugin: [dem] contact, adhesion, rolling and twisting
// models (crates/dem_granular/src/contact.rs:52-91).
struct HertzMindlinContactPlugin : Plugin {
    std::string name() const override { return "HertzMindlinContactPlugin"; }
    std::vector<std::string> provides() const override { return {"contact_forces"}; }
    std::vector<std::string> requires_() const override { return {"dem_particles", "neighbor_list"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* dem = section(a, "dem");
            auto pick = [&](const char* key, const char* d0, const char* d1, int& out) {
                const std::string v = text(dem, key, d0);
                if (v != d0 && v != d1) throw ConfigError(std::string(key) + " = \"" + v + "\": " + d0 + " or " + d1);
                out = v == d0 ? 0 : 1;
            };
            pick("contact_model", "hertz", "hooke", a.cfg.contact_model);
            pick("adhesion_model", "jkr", "dmt", a.cfg.adhesion_model);
            pick("rolling_model", "constant", "sds", a.cfg.rolling_model);
            pick("twisting_model", "constant", "sds", a.cfg.twisting_model);
        });
    }
};

// solid-sphere mass and inverse inertia (crates/dem_atom/src/insert.rs:343-349)
double sphere_mass(double density, double r) { return ((density * 4.0) / 3.0) * kPi * ((r * r) * r); }
double sphere_inv_inertia(double m, double r) { return 1.0 / (((0.4 * m) * r) * r); }

void push_sphere(HostState& h, const double* x, const double* v, double r, double density, uint32_t type) {
    const double m = sphere_mass(density, r);
    h.tag.push_back((uint32_t)h.tag.size());
    h.type.push_back(type);
    h.pos.insert(h.pos.end(), x, x + 3);
    h.vel.insert(h.vel.end(), v, v + 3);
    h.mass.push_back(m);
    h.cutoff_radius.push_back(r);
    h.radius.push_back(r);
    h.density.push_back(density);
    h.inv_inertia.push_back(sphere_inv_inertia(m, r));
    h.omega.insert(h.omega.end(), {0.0, 0.0, 0.0});
    h.quat.insert(h.quat.end(), {1.0, 0.0, 0.0, 0.0});
}

// the reference's CSV particle file: x,y,z,radius,vx,vy,vz[,type], an
// optional header line, '#' comments (crates/dem_atom/src/insert.rs:652-776)
void read_csv(HostState& h, const std::string& path, double density) {
    std::ifstream f(path);
    if (!f) throw ConfigError("cannot read " + path);
    std::string line;
    int ln = 0;
    while (std::getline(f, line)) {
        const int this_ln = ln++;
        const size_t b = line.find_first_not_of(" \t\r");
        if (b == std::string::npos || line[b] == '#') continue;
        if (this_ln == 0 && std::isalpha((unsigned char)line[b])) continue;
        std::vector<double> c;
        std::stringstream ss(line);
        std::string cell;
        while (std::getline(ss, cell, ',')) c.push_back(std::stod(cell));
        if (c.size() < 4) throw ConfigError(path + ": a row needs x,y,z,radius");
        const double v[3] = {c.size() >= 7 ? c[4] : 0.0, c.size() >= 7 ? c[5] : 0.0, c.size() >= 7 ? c[6] : 0.0};
        push_sphere(h, c.data(), v, c[3], density, c.size() > 7 ? (uint32_t)c[7] : 0u);
    }
}

// Rayleigh-wave timestep, 0.15 of the smallest sphere's (calculate_delta_time,
// crates/dem_atom/src/insert.rs:1392-1431)
double rayleigh_dt(double r, double density, double E, double nu) {
    const double g = E / (2.0 * (1.0 + nu));
    const double alpha = 0.1631 * nu + 0.876605;
    return 0.15 * (kPi * r / alpha * std::sqrt(density / g));
}

// [gpu] generate = "device" for a granular config: one random insertion block
// in the domain (inset by the radius), made by mdg_generate_gas with the same
// rejection rule (1.1 (r_i + r_j)) and Gaussian components of std `velocity`;
// block regions, files, several blocks and directional velocities stay on the
// host generator.  dt from the smallest radius the block allows.
void device_gas(App& a, const std::vector<const toml::Table*>& blocks) {
    if (blocks.size() != 1) throw ConfigError("generate = \"device\": one [[particles.insert]] block");
    const toml::Table* b = blocks[0];
    if (text(b, "source", "random") != "random" || toml::find(*b, "rate") || toml::find(*b, "region"))
        throw ConfigError("generate = \"device\": random insertion in the whole domain only");
    for (const char* k : {"velocity_x", "velocity_y", "velocity_z"})
        if (num(b, k, 0.0) != 0.0) throw ConfigError(std::string("generate = \"device\": ") + k + " is not supported");
    const long long n = integer(b, "count", -1);
    if (n < 1) throw ConfigError("[[particles.insert]] needs count");
    mdg_gas_spec g{};
    g.n = (size_t)n;
    const toml::Value* rv = toml::find(*b, "radius");
    if (!rv) throw ConfigError("[[particles.insert]] needs radius");
    if (rv->kind == toml::Value::TABLE) {
        if (text(rv->t.get(), "distribution", "") != "uniform") throw ConfigError("radius distribution: fixed or uniform only");
        g.rmin = num(rv->t.get(), "min", 0.0);
        g.rmax = num(rv->t.get(), "max", 0.0);
    } else {
        g.rmin = g.rmax = rv->number();
    }
    g.density = num(b, "density", 2500.0);
    g.sep_factor = 1.1;
    g.inset = 1;
    g.velocity_mode = MDG_VEL_GAUSSIAN;
    g.speed = num(b, "velocity", 0.0);
    const std::string mat = text(b, "material", a.material_names[0]);
    size_t mi = 0;
    while (mi < a.material_names.size() && a.material_names[mi] != mat) mi++;
    if (mi == a.material_names.size()) throw ConfigError("material \"" + mat + "\" is not in [[dem.materials]]");
    g.material = (uint32_t)mi;
    g.seed = a.opts.seed;
    a.device_gen_n = (size_t)n;
    a.device_gen_density = g.density;
    a.device_gen = [g](App& app) {
        size_t placed = 0;
        return mdg_generate_gas(app.ctx, 0, &g, &placed);
    };
    if (a.cfg.dt == 0.0)
        a.cfg.dt = rayleigh_dt(g.rmin, g.density, a.materials[0].youngs_mod, a.materials[0].poisson_ratio);
}

// DemAtomInsertPlugin: [[particles.insert]] (crates/dem_atom/src/insert.rs:
// 417-614): random insertion in the domain inset by the radius or in a block
// region, rejection at 1.1 (r_i + r_j) (mdg_rsa_spheres), Gaussian velocity
// components of std `velocity` plus velocity_x/y/z; or a CSV file.
struct DemAtomInsertPlugin : Plugin {
    std::string name() const override { return "DemAtomInsertPlugin"; }
    std::vector<std::string> requires_() const override { return {"dem_particles"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::PostSetup, [](App& a) {
            const toml::Table* parts = section(a, "particles");
            std::vector<const toml::Table*> blocks;
            if (parts) blocks = table_array(*parts, "insert");
            if (blocks.empty()) throw ConfigError("a DEM config needs [[particles.insert]]");
            HostState& h = a.state;
            h = HostState{};
            h.dem = true;
            if (a.gen_device) {
                device_gas(a, blocks);
                return;
            }
            double rmin_all = std::numeric_limits<double>::infinity(), dmax = 0.0;
            for (size_t k = 0; k < blocks.size(); k++) {
                const toml::Table* b = blocks[k];
                const double density = num(b, "density", 2500.0);
                dmax = std::fmax(dmax, density);
                if (text(b, "source", "random") == "file") {
                    if (text(b, "format", "csv") != "csv") throw ConfigError("insert source format: only csv");
                    const size_t n0 = h.size();
                    read_csv(h, text(b, "file", ""), density);
                    for (size_t i = n0; i < h.size(); i++) rmin_all = std::fmin(rmin_all, h.radius[i]);
                    continue;
                }
                if (toml::find(*b, "rate")) throw ConfigError("rate-based insertion is not supported");
                const long long n = integer(b, "count", -1);
                if (n < 0) throw ConfigError("[[particles.insert]] needs count");
                double rmin, rmax;
                const toml::Value* rv = toml::find(*b, "radius");
                if (!rv) throw ConfigError("[[particles.insert]] needs radius");
                if (rv->kind == toml::Value::TABLE) {
                    if (text(rv->t.get(), "distribution", "") != "uniform")
                        throw ConfigError("radius distribution: fixed or uniform only");
                    rmin = num(rv->t.get(), "min", 0.0);
                    rmax = num(rv->t.get(), "max", 0.0);
                } else {
                    rmin = rmax = rv->number();
                }
                double lo[3], hi[3];
                int inset = 1;
                for (int d = 0; d < 3; d++) {
                    lo[d] = a.cfg.box_lo[d];
                    hi[d] = a.cfg.box_hi[d];
                }
                if (const toml::Value* reg = toml::find(*b, "region")) {
                    // Region::Block: centres uniform inside [min, max], no inset
                    if (reg->kind != toml::Value::TABLE || text(reg->t.get(), "type", "") != "block")
                        throw ConfigError("insertion region: only block regions are supported");
                    const toml::Value* mn = toml::find(*reg->t, "min");
                    const toml::Value* mx = toml::find(*reg->t, "max");
                    if (!mn || !mx || mn->array().size() != 3 || mx->array().size() != 3)
                        throw ConfigError("block region needs min and max of 3 numbers");
                    for (int d = 0; d < 3; d++) {
                        lo[d] = mn->array()[d].number();
                        hi[d] = mx->array()[d].number();
                    }
                    inset = 0;
                }
                std::vector<double> pos((size_t)n * 3), rad((size_t)n);
                size_t placed = 0;
                const int st = mdg_rsa_spheres((size_t)n, lo, hi, rmin, rmax, 1.1, inset, a.opts.seed + k, 0,
                                               pos.data(), rad.data(), &placed);
                if (st != MDG_OK)
                    throw ConfigError("insertion placed " + std::to_string(placed) + " of " + std::to_string(n));
                const std::string mat = text(b, "material", a.material_names[0]);
                size_t mi = 0;
                while (mi < a.material_names.size() && a.material_names[mi] != mat) mi++;
                if (mi == a.material_names.size()) throw ConfigError("material \"" + mat + "\" is not in [[dem.materials]]");
                const double sd = num(b, "velocity", 0.0);
                const double v0[3] = {num(b, "velocity_x", 0.0), num(b, "velocity_y", 0.0), num(b, "velocity_z", 0.0)};
                std::mt19937_64 gen(a.opts.seed + 7919ull * (k + 1));
                std::normal_distribution<double> nd(0.0, sd > 0.0 ? sd : 1.0);
                for (long long i = 0; i < n; i++) {
                    double v[3];
                    for (int d = 0; d < 3; d++) v[d] = (sd > 0.0 ? nd(gen) : 0.0) + v0[d];
                    push_sphere(h, &pos[3 * i], v, rad[i], density, (uint32_t)mi);
                    rmin_all = std::fmin(rmin_all, rad[i]);
                }
            }
            if (a.cfg.dt == 0.0)
                a.cfg.dt = rayleigh_dt(rmin_all, dmax, a.materials[0].youngs_mod, a.materials[0].poisson_ratio);
        });
    }
};

// The integrators and the granular temperature run inside the device step;
// these plugins keep the group's composition and provide/require checks.
struct NamedPlugin : Plugin {
    std::string n;
    std::vector<std::string> p, r;
    NamedPlugin(std::string name, std::vector<std::string> prov, std::vector<std::string> req)
        : n(std::move(name)), p(std::move(prov)), r(std::move(req)) {}
    std::string name() const override { return n; }
    std::vector<std::string> provides() const override { return p; }
    std::vector<std::string> requires_() const override { return r; }
    void build(App&) override {}
};

// WallPlugin: [[wall]] plane walls (crates/dem_wall/src/lib.rs:160-262).
struct WallPlugin : Plugin {
    std::string name() const override { return "WallPlugin"; }
    std::vector<std::string> requires_() const override { return {"dem_particles"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            for (const toml::Table* w : table_array(a.input, "wall")) {
                check_keys("wall", *w,
                           {"type", "point_x", "point_y", "point_z", "normal_x", "normal_y", "normal_z", "material",
                            "name", "bound_x_low", "bound_x_high", "bound_y_low", "bound_y_high", "bound_z_low",
                            "bound_z_high", "velocity", "oscillate", "servo", "axis", "center", "radius", "lo", "hi",
                            "inside", "region", "temperature"});
                if (text(w, "type", "plane") != "plane") throw ConfigError("the GPU path supports plane walls only");
                if (toml::find(*w, "oscillate") || toml::find(*w, "servo"))
                    throw ConfigError("oscillating and servo walls are not supported by the GPU path");
                if (toml::find(*w, "temperature")) throw ConfigError("wall heat transfer is not supported by the GPU path");
                const std::string mat = text(w, "material", "");
                size_t mi = 0;
                while (mi < a.material_names.size() && a.material_names[mi] != mat) mi++;
                if (mi == a.material_names.size())
                    throw ConfigError("wall material \"" + mat + "\" is not in [[dem.materials]]");
                mdg_wall x{};
                const char* ax = "xyz";
                for (int d = 0; d < 3; d++) {
                    const std::string c(1, ax[d]);
                    x.point[d] = num(w, "point_" + c, 0.0);
                    x.normal[d] = num(w, "normal_" + c, 0.0);
                    x.bound_lo[d] = num(w, "bound_" + c + "_low", -std::numeric_limits<double>::infinity());
                    x.bound_hi[d] = num(w, "bound_" + c + "_high", std::numeric_limits<double>::infinity());
                }
                if (const toml::Value* v = toml::find(*w, "velocity")) {
                    if (v->array().size() != 3) throw ConfigError("wall velocity needs 3 numbers");
                    for (int d = 0; d < 3; d++) x.velocity[d] = v->array()[d].number();
                }
                x.material = (int)mi;
                a.walls.push_back(x);
            }
        });
    }
};

// ---------------------------------------------------------------------------
// LJ group
// ---------------------------------------------------------------------------

// LatticePlugin: [lattice] FCC (crates/md_lattice/src/lib.rs:232-471): lattice
// constant (4/rho)^(1/3), n = floor(L / a) cells stretched to the box, 4-atom
// basis, Gaussian velocities with the centre-of-mass velocity removed and
// rescaled to exactly T with 3N - 3 degrees of freedom; dt = 0.005 unless set.
struct LatticePlugin : Plugin {
    std::string name() const override { return "LatticePlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::PostSetup, [](App& a) {
            const toml::Table* lat = section(a, "lattice");
            if (!lat || text(lat, "style", "fcc") != "fcc") throw ConfigError("an LJ config needs [lattice] style = \"fcc\"");
            check_keys("lattice", *lat,
                       {"style", "density", "temperature", "mass", "skin", "type_fractions", "type_masses"});
            const double rho = num(lat, "density", 0.85), T = num(lat, "temperature", 0.85);
            const double mass = num(lat, "mass", 1.0), skin = num(lat, "skin", 1.25);
            std::vector<double> fractions = numbers(lat, "type_fractions"), tmass = numbers(lat, "type_masses");
            if (fractions.empty()) fractions.push_back(1.0);
            const double L = a.cfg.box_hi[0] - a.cfg.box_lo[0], lo = a.cfg.box_lo[0];
            const int nc = (int)std::floor(L / std::pow(4.0 / rho, 1.0 / 3.0));
            if (nc < 1) throw ConfigError("[lattice] density leaves no FCC cell in the box");
            const double ax = L / nc;
            const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
            HostState& h = a.state;
            h = HostState{};
            h.dem = false;
            if (a.gen_device) {  // mdg_generate_fcc: the same lattice, types and masses, T fixed on the device
                if ((int)fractions.size() > MDG_GEN_MAX_TYPES) throw ConfigError("[lattice] more than 8 types");
                if (a.lj_types > 1 && (int)fractions.size() > a.lj_types)
                    throw ConfigError("[lattice] type_fractions give more types than [lj] types");
                mdg_fcc_spec f{};
                f.density = rho;
                f.temperature = T;
                f.mass = mass;
                f.skin = skin;
                f.seed = a.opts.seed;
                f.n_types = (int32_t)fractions.size();
                for (size_t q = 0; q < fractions.size(); q++) {
                    f.type_fractions[q] = fractions[q];
                    f.type_masses[q] = q < tmass.size() ? tmass[q] : 0.0;
                }
                long long n = 4;
                for (int d = 0; d < 3; d++)
                    n *= (long long)std::floor((a.cfg.box_hi[d] - a.cfg.box_lo[d]) / std::cbrt(4.0 / rho));
                a.device_gen_n = (size_t)n;
                a.device_gen = [f](App& app) {
                    size_t made = 0;
                    return mdg_generate_fcc(app.ctx, 0, &f, &made);
                };
                if (a.cfg.dt == 0.0) a.cfg.dt = 0.005;
                return;
            }
            std::mt19937_64 gen(a.opts.seed);
            std::normal_distribution<double> nd(0.0, std::sqrt(T / mass)), n01(0.0, 1.0);
            // types by index (fcc_insert, md_lattice/src/lib.rs:291-327): the
            // first cumulative fraction above (k + 0.5) / n, else the last type
            const size_t total = (size_t)4 * nc * nc * nc;
            for (int ix = 0; ix < nc; ix++)
                for (int iy = 0; iy < nc; iy++)
                    for (int iz = 0; iz < nc; iz++)
                        for (int b = 0; b < 4; b++) {
                            const double f = ((double)h.tag.size() + 0.5) / (double)total;
                            uint32_t t = (uint32_t)fractions.size() - 1;
                            for (size_t q = 0; q < fractions.size(); q++)
                                if (f < fractions[q]) {
                                    t = (uint32_t)q;
                                    break;
                                }
                            const double m = tmass.empty() ? mass : (t < tmass.size() ? tmass[t] : mass);
                            if (!(m > 0.0)) throw ConfigError("[lattice] masses must be positive");
                            h.tag.push_back((uint32_t)h.tag.size());
                            h.type.push_back(t);
                            h.pos.push_back(lo + (ix + basis[b][0]) * ax);
                            h.pos.push_back(lo + (iy + basis[b][1]) * ax);
                            h.pos.push_back(lo + (iz + basis[b][2]) * ax);
                            for (int d = 0; d < 3; d++)
                                h.vel.push_back(tmass.empty() ? nd(gen) : n01(gen) * std::sqrt(T / m));
                            h.mass.push_back(m);
                            h.cutoff_radius.push_back(skin);
                        }
            if (a.lj_types > 1 && (int)fractions.size() > a.lj_types)
                throw ConfigError("[lattice] type_fractions give more types than [lj] types");
            const size_t n = h.size();
            double vs[3] = {0, 0, 0};
            for (size_t i = 0; i < n; i++)
                for (int d = 0; d < 3; d++) vs[d] += h.vel[3 * i + d];
            for (size_t i = 0; i < n; i++)
                for (int d = 0; d < 3; d++) h.vel[3 * i + d] -= vs[d] / (double)n;
            double ke = 0.0;
            for (size_t i = 0; i < n; i++)
                ke += h.mass[i] * (h.vel[3 * i] * h.vel[3 * i] + h.vel[3 * i + 1] * h.vel[3 * i + 1] +
                                   h.vel[3 * i + 2] * h.vel[3 * i + 2]);
            const double cur = ke / (3.0 * (double)n - 3.0);
            if (cur > 1e-20)
                for (double& v : h.vel) v *= std::sqrt(T / cur);
            if (a.cfg.dt == 0.0) a.cfg.dt = 0.005;
        });
    }
};

// LJForcePlugin: [lj] (LJConfig, crates/md_lj/src/lib.rs:115-184) and
// build_lj_pair_table (lib.rs:334-384): one type from epsilon / sigma, or
// with [[lj.types]] the n x n table, cross pairs by the mixing rule
// (arithmetic means for "arithmetic", else geometric) at the global cutoff,
// then the [[lj.pair_coeffs]] overrides set (a, b) and (b, a) in order.
struct LJForcePlugin : Plugin {
    std::string name() const override { return "LJForcePlugin"; }
    std::vector<std::string> requires_() const override { return {"neighbor_list"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* lj = section(a, "lj");
            if (lj) check_keys("lj", *lj, {"epsilon", "sigma", "cutoff", "mixing", "types", "pair_coeffs"});
            a.cfg.lj_epsilon = num(lj, "epsilon", 1.0);
            a.cfg.lj_sigma = num(lj, "sigma", 1.0);
            a.cfg.lj_cutoff = num(lj, "cutoff", 2.5);
            if (!lj || !toml::find(*lj, "types")) return;
            std::vector<std::pair<double, double>> types;
            for (const toml::Table* t : table_array(*lj, "types")) {
                check_keys("lj.types", *t, {"epsilon", "sigma"});
                if (!toml::find(*t, "epsilon") || !toml::find(*t, "sigma"))
                    throw ConfigError("[[lj.types]] needs epsilon and sigma");
                types.emplace_back(num(t, "epsilon", 0.0), num(t, "sigma", 0.0));
            }
            if (types.empty()) throw ConfigError("[lj] types is empty");
            const toml::Value* mix = toml::find(*lj, "mixing");
            const bool arith = mix && mix->kind == toml::Value::STRING && mix->s == "arithmetic";
            const size_t n = types.size();
            const double cut = a.cfg.lj_cutoff;
            std::vector<mdg_lj_pair> tab(n * n);
            for (size_t i = 0; i < n; i++)
                for (size_t j = i; j < n; j++) {
                    const double ei = types[i].first, si = types[i].second;
                    const double ej = types[j].first, sj = types[j].second;
                    const double eps = arith ? (ei + ej) / 2.0 : std::sqrt(ei * ej);
                    const double sig = arith ? (si + sj) / 2.0 : std::sqrt(si * sj);
                    tab[i * n + j] = tab[j * n + i] = mdg_lj_pair{eps, sig, cut};
                }
            for (const toml::Table* o : table_array(*lj, "pair_coeffs")) {
                check_keys("lj.pair_coeffs", *o, {"types", "epsilon", "sigma", "cutoff"});
                const toml::Value* tv = toml::find(*o, "types");
                if (!tv || tv->kind != toml::Value::ARRAY || tv->array().size() != 2 || !toml::find(*o, "epsilon") ||
                    !toml::find(*o, "sigma"))
                    throw ConfigError("[[lj.pair_coeffs]] needs types = [a, b], epsilon and sigma");
                const long long ta = tv->array()[0].integer(), tb = tv->array()[1].integer();
                if (ta < 0 || tb < 0 || ta >= (long long)n || tb >= (long long)n)
                    throw ConfigError("[[lj.pair_coeffs]] types = [" + std::to_string(ta) + ", " + std::to_string(tb) +
                                      "]: only " + std::to_string(n) + " types");
                const mdg_lj_pair q{num(o, "epsilon", 0.0), num(o, "sigma", 0.0), num(o, "cutoff", cut)};
                tab[(size_t)ta * n + (size_t)tb] = tab[(size_t)tb * n + (size_t)ta] = q;
            }
            if (n == 1) {  // one type: lj_force reads the 1 x 1 table
                a.cfg.lj_epsilon = tab[0].epsilon;
                a.cfg.lj_sigma = tab[0].sigma;
                a.cfg.lj_cutoff = tab[0].cutoff;
            } else {
                a.lj_types = (int)n;
                a.lj_pairs = tab;
            }
        });
    }
};

// NoseHooverPlugin: [thermostat] (crates/md_thermostat/src/lib.rs:85-97).
struct NoseHooverPlugin : Plugin {
    std::string name() const override { return "NoseHooverPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* th = section(a, "thermostat");
            if (!th) return;
            check_keys("thermostat", *th, {"temperature", "coupling", "group"});
            if (toml::find(*th, "group")) throw ConfigError("thermostat groups are not supported by the GPU path");
            a.cfg.nose_hoover = 1;
            a.cfg.nh_temperature = num(th, "temperature", 0.85);
            a.cfg.nh_coupling = num(th, "coupling", 1.0);
        });
    }
};

// LangevinPlugin: [langevin] (crates/md_thermostat/src/lib.rs:380-581).
struct LangevinPlugin : Plugin {
    std::string name() const override { return "LangevinPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* lv = section(a, "langevin");
            if (!lv) return;
            check_keys("langevin", *lv, {"temperature", "damping", "seed", "group"});
            if (toml::find(*lv, "group")) throw ConfigError("thermostat groups are not supported by the GPU path");
            a.cfg.langevin = 1;
            a.cfg.lv_temperature = num(lv, "temperature", 0.85);
            a.cfg.lv_damping = num(lv, "damping", 1.0);
            a.cfg.lv_seed = (uint64_t)integer(lv, "seed", 12345);
        });
    }
};

// MeasurePlugin: [measure] RDF and MSD sampling (md_measure/src/lib.rs:333-600),
// written to <output dir>/rdf.txt and msd.txt at the end of the run.
struct MeasurePlugin : Plugin {
    struct Acc {
        long long rdf_every = 0, msd_every = 0;
        int bins = 200;
        double rmax = 3.0;
        std::vector<double> g;
        int samples = 0;
        std::vector<std::pair<long long, double>> msd;
    };
    std::shared_ptr<Acc> acc = std::make_shared<Acc>();
    std::string name() const override { return "MeasurePlugin"; }
    void build(App& app) override {
        auto c = acc;
        app.add_setup_system(Schedule::Setup, [c](App& a) {
            const toml::Table* m = section(a, "measure");
            if (!m) return;
            c->rdf_every = integer(m, "rdf_interval", 0);
            c->msd_every = integer(m, "msd_interval", 0);
            c->bins = (int)integer(m, "rdf_bins", 200);
            c->rmax = num(m, "rdf_cutoff", 3.0);
            if (c->rdf_every > 0) a.intervals.push_back(c->rdf_every);
            if (c->msd_every > 0) a.intervals.push_back(c->msd_every);
        });
        app.add_update_system(Schedule::LastOutput, [c](App& a) {
            if (a.done() == 0) {
                if (c->msd_every > 0 && mdg_msd_reset(a.ctx, 0) != MDG_OK) throw ConfigError("msd reset failed");
                return;
            }
            if (c->rdf_every > 0 && a.done() % c->rdf_every == 0) {
                std::vector<uint64_t> counts((size_t)c->bins);
                if (mdg_rdf(a.ctx, 0, c->rmax, c->bins, counts.data()) != MDG_OK) throw ConfigError("rdf failed");
                // g_k = counts_k V / (N (N - 1) / 2 shell_k) (md_measure/src/lib.rs:420-440)
                const double n = (double)a.state.size();
                double vol = 1.0;
                for (int d = 0; d < 3; d++) vol *= a.cfg.box_hi[d] - a.cfg.box_lo[d];
                const double dr = c->rmax / c->bins;
                if (c->g.empty()) c->g.assign((size_t)c->bins, 0.0);
                for (int k = 0; k < c->bins; k++) {
                    const double r0 = k * dr, r1 = (k + 1) * dr;
                    const double shell = 4.0 / 3.0 * kPi * (r1 * r1 * r1 - r0 * r0 * r0);
                    c->g[k] += (double)counts[k] * vol / (n * (n - 1.0) / 2.0 * shell);
                }
                c->samples++;
            }
            if (c->msd_every > 0 && a.done() % c->msd_every == 0) {
                double v = 0.0;
                if (mdg_msd(a.ctx, 0, &v) != MDG_OK) throw ConfigError("msd failed");
                c->msd.emplace_back(a.step, v);
            }
        });
        app.finish.push_back([c](App& a) {
            if (c->samples == 0 && c->msd.empty()) return;
            std::filesystem::create_directories(a.out_dir);
            if (c->samples) {
                std::ofstream f(a.out_dir + "/rdf.txt");
                const double dr = c->rmax / c->bins;
                char buf[64];
                for (int k = 0; k < c->bins; k++) {
                    std::snprintf(buf, sizeof(buf), "%.6f %.6f\n", (k + 0.5) * dr, c->g[k] / c->samples);
                    f << buf;
                }
            }
            if (!c->msd.empty()) {
                std::ofstream f(a.out_dir + "/msd.txt");
                char buf[64];
                for (auto& e : c->msd) {
                    std::snprintf(buf, sizeof(buf), "%lld %.10e\n", e.first, e.second);
                    f << buf;
                }
            }
        });
    }
};

std::string restart_dir(const App& a) { return a.out_dir + "/restart"; }

// RestartPlugin: [restart] interval, format, read (RestartConfig and the
// restart output, crates/mddem_print/src/lib.rs:267-277, 1050-1066):
// restart_{step}_rank0.bin (bincode) or .json in <output>/restart
// (restart_base_dir, lib.rs:528-534) every `interval` steps; `read` resumes
// from the latest of them in the configured format (resume_from_restart).
struct RestartPlugin : Plugin {
    std::string name() const override { return "RestartPlugin"; }
    void build(App& app) override {
        auto every = std::make_shared<long long>(0);
        app.add_setup_system(Schedule::Setup, [every](App& a) {
            const toml::Table* r = section(a, "restart");
            if (!r) return;
            check_keys("restart", *r, {"interval", "format", "read"});
            *every = integer(r, "interval", 0);
            // write_restart_inner (lib.rs:1050-1070): "json", anything else bincode
            a.restart_json = text(r, "format", "bincode") == "json";
            a.restart_read = boolean(r, "read", false);
            if (*every > 0) a.intervals.push_back(*every);
        });
        app.add_update_system(Schedule::LastOutput, [every](App& a) {
            if (*every <= 0 || a.done() == 0 || a.done() % *every != 0) return;
            const size_t n = a.state.size();
            HostState d;
            d.dem = a.state.dem;
            d.tag.resize(n);
            d.type.resize(n);
            d.pos.resize(3 * n);
            d.vel.resize(3 * n);
            d.mass.resize(n);
            d.cutoff_radius.resize(n);
            std::vector<double> force(3 * n), torque(3 * n), density;
            std::vector<int32_t> image(3 * n);
            mdg_state_view v{};
            v.n = n;
            v.tag = d.tag.data();
            v.type = d.type.data();
            v.pos = d.pos.data();
            v.vel = d.vel.data();
            v.force = force.data();
            v.mass = d.mass.data();
            v.cutoff_radius = d.cutoff_radius.data();
            v.image = image.data();
            if (d.dem) {
                d.radius.resize(n);
                d.inv_inertia.resize(n);
                d.omega.resize(3 * n);
                d.quat.resize(4 * n);
                v.radius = d.radius.data();
                v.inv_inertia = d.inv_inertia.data();
                v.omega = d.omega.data();
                v.torque = torque.data();
                v.quat = d.quat.data();
            }
            int st = mdg_download_state(a.ctx, 0, &v);
            if (st != MDG_OK) throw ConfigError(std::string("mdg_download_state: ") + mdg_status_string(st));
            std::vector<uint32_t> keys;
            std::vector<double> vals;
            RestartInput in;
            in.state = &d;
            in.force = &force;
            in.step = (uint64_t)a.step;
            in.dt = a.cfg.dt;
            if (d.dem) {
                in.torque = &torque;
                // densities by tag (the device keeps no density)
                std::unordered_map<uint32_t, double> by_tag;
                for (size_t i = 0; i < n; i++) by_tag[a.state.tag[i]] = a.state.density[i];
                density.resize(n);
                for (size_t i = 0; i < n; i++) density[i] = by_tag.at(d.tag[i]);
                in.density = &density;
                size_t nh = 0;
                st = mdg_get_history(a.ctx, 0, nullptr, nullptr, 0, &nh);
                if (st != MDG_OK) throw ConfigError(std::string("mdg_get_history: ") + mdg_status_string(st));
                keys.resize(2 * nh);
                vals.resize(7 * nh);
                if (nh) st = mdg_get_history(a.ctx, 0, keys.data(), vals.data(), nh, &nh);
                if (st != MDG_OK) throw ConfigError(std::string("mdg_get_history: ") + mdg_status_string(st));
                keys.resize(2 * nh);
                vals.resize(7 * nh);
                in.hist_keys = &keys;
                in.hist_vals = &vals;
            }
            const std::string dir = restart_dir(a);
            std::filesystem::create_directories(dir);
            const std::string path = dir + "/" + restart_filename((uint64_t)a.step, 0, a.restart_json);
            std::ofstream f(path, std::ios::binary);
            f << (a.restart_json ? restart_json(in) : restart_bincode(in));
            if (!f) throw ConfigError("cannot write " + path);
        });
    }
};

void json_num(std::ostringstream& o, double x) {
    if (std::isinf(x)) {
        o << (x > 0 ? "\"inf\"" : "\"-inf\"");
        return;
    }
    char b[40];
    std::snprintf(b, sizeof(b), "%.17g", x);
    o << b;
}

void json_vec(std::ostringstream& o, const double* x, int n) {
    o << "[";
    for (int k = 0; k < n; k++) {
        if (k) o << ", ";
        json_num(o, x[k]);
    }
    o << "]";
}

}  // namespace

void add_granular_plugins(App& app) {
    app.dem = true;
    app.cfg.kind = MDG_KIND_DEM;
    app.add_plugin(std::make_unique<DemAtomPlugin>());
    app.add_plugin(std::make_unique<DemAtomInsertPlugin>());
    app.add_plugin(std::make_unique<NamedPlugin>("VelocityVerletPlugin", std::vector<std::string>{},
                                                 std::vector<std::string>{}));
    app.add_plugin(std::make_unique<HertzMindlinContactPlugin>());
    app.add_plugin(std::make_unique<NamedPlugin>("RotationalDynamicsPlugin", std::vector<std::string>{},
                                                 std::vector<std::string>{"dem_particles"}));
    app.add_plugin(std::make_unique<NamedPlugin>("GranularTempPlugin", std::vector<std::string>{},
                                                 std::vector<std::string>{"dem_particles"}));
}

void add_lj_plugins(App& app) {
    app.dem = false;
    app.cfg.kind = MDG_KIND_LJ;
    app.add_plugin(std::make_unique<LatticePlugin>());
    app.add_plugin(std::make_unique<LJForcePlugin>());
    app.add_plugin(std::make_unique<NoseHooverPlugin>());
    app.add_plugin(std::make_unique<MeasurePlugin>());
}

void add_wall_plugin(App& app) { app.add_plugin(std::make_unique<WallPlugin>()); }
void add_restart_plugin(App& app) { app.add_plugin(std::make_unique<RestartPlugin>()); }

Resumed resume_from_restart(App& a) {
    Resumed out;
    const std::string dir = restart_dir(a);
    const std::string path = latest_restart(dir, a.restart_json);
    if (path.empty()) {
        std::printf("# Restart: no restart files found in %s\n", dir.c_str());
        return out;
    }
    std::printf("# Restart: reading from %s\n", path.c_str());
    std::ifstream f(path, std::ios::binary);
    const std::string bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (!f.good() && !f.eof()) throw ConfigError("cannot read " + path);
    RestartRead r = a.restart_json ? restart_read_json(bytes) : restart_read(bytes);
    if (r.state.dem != a.dem)
        throw ConfigError(path + (a.dem ? ": no DemAtom buffer for a granular run" : ": a DEM file for an LJ run"));
    a.state = std::move(r.state);
    a.first_step = (long long)r.step;
    out.force = std::move(r.force);
    out.torque = std::move(r.torque);
    out.hist_keys = std::move(r.hist_keys);
    out.hist_vals = std::move(r.hist_vals);
    std::printf("# Restart: loaded %zu atoms from step %llu\n", a.state.size(), (unsigned long long)r.step);
    return out;
}

void write_initial_restart(const App& a, const std::string& path) {
    RestartInput in;
    in.state = &a.state;
    in.density = a.state.dem ? &a.state.density : nullptr;
    in.dt = a.cfg.dt;
    const bool json = path.size() >= 5 && path.compare(path.size() - 5, 5, ".json") == 0;
    std::ofstream f(path, std::ios::binary);
    f << (json ? restart_json(in) : restart_bincode(in));
    if (!f) throw ConfigError("cannot write " + path);
}
void add_langevin_plugin(App& app) { app.add_plugin(std::make_unique<LangevinPlugin>()); }

std::string config_json(const App& a) {
    const mdg_config& c = a.cfg;
    std::ostringstream o;
    o << "{\"kind\": " << c.kind << ", \"precision\": " << c.precision << ", \"box_lo\": ";
    json_vec(o, c.box_lo, 3);
    o << ", \"box_hi\": ";
    json_vec(o, c.box_hi, 3);
    o << ", \"dt\": ";
    json_num(o, c.dt);
    o << ", \"skin_fraction\": ";
    json_num(o, c.skin_fraction);
    o << ", \"bin_size\": ";
    json_num(o, c.bin_size);
    o << ", \"every\": " << c.every << ", \"check\": " << c.check << ", \"sort_every\": " << c.sort_every
      << ", \"newton\": " << c.newton << ", \"n_materials\": " << c.n_materials << ", \"materials\": [";
    for (int k = 0; k < c.n_materials; k++) {
        const double* m = &c.materials[k].youngs_mod;
        if (k) o << ", ";
        json_vec(o, m, 14);
    }
    o << "], \"contact_model\": " << c.contact_model << ", \"adhesion_model\": " << c.adhesion_model
      << ", \"rolling_model\": " << c.rolling_model << ", \"twisting_model\": " << c.twisting_model
      << ", \"lj_epsilon\": ";
    json_num(o, c.lj_epsilon);
    o << ", \"lj_sigma\": ";
    json_num(o, c.lj_sigma);
    o << ", \"lj_cutoff\": ";
    json_num(o, c.lj_cutoff);
    o << ", \"nose_hoover\": " << c.nose_hoover << ", \"nh_temperature\": ";
    json_num(o, c.nh_temperature);
    o << ", \"nh_coupling\": ";
    json_num(o, c.nh_coupling);
    o << ", \"virial\": " << c.virial << ", \"rebuild_policy\": " << c.rebuild_policy
      << ", \"threads_per_particle\": " << c.threads_per_particle << ", \"neighbor_capacity\": " << c.neighbor_capacity
      << ", \"history_capacity\": " << c.history_capacity << ", \"langevin\": " << c.langevin
      << ", \"lv_temperature\": ";
    json_num(o, c.lv_temperature);
    o << ", \"lv_damping\": ";
    json_num(o, c.lv_damping);
    o << ", \"lv_seed\": " << c.lv_seed << ", \"fixed\": [" << c.fixed[0] << ", " << c.fixed[1] << ", " << c.fixed[2]
      << "], \"n_lj_types\": " << c.n_lj_types << ", \"lj_pairs\": [";
    for (int k = 0; c.lj_pairs && k < c.n_lj_types * c.n_lj_types; k++) {
        if (k) o << ", ";
        json_vec(o, &c.lj_pairs[k].epsilon, 3);
    }
    o << "], \"walls\": [";
    for (int k = 0; k < c.n_walls; k++) {
        const mdg_wall& w = c.walls[k];
        if (k) o << ", ";
        o << "{\"point\": ";
        json_vec(o, w.point, 3);
        o << ", \"normal\": ";
        json_vec(o, w.normal, 3);
        o << ", \"bound_lo\": ";
        json_vec(o, w.bound_lo, 3);
        o << ", \"bound_hi\": ";
        json_vec(o, w.bound_hi, 3);
        o << ", \"velocity\": ";
        json_vec(o, w.velocity, 3);
        o << ", \"material\": " << w.material << "}";
    }
    const HostState& h = a.state;
    double ps[3] = {0, 0, 0}, rs = 0.0, ms = 0.0;
    long long ts = 0;
    for (size_t i = 0; i < h.size(); i++) {
        ts += h.type[i];
        for (int d = 0; d < 3; d++) ps[d] += h.pos[3 * i + d];
        ms += h.mass[i];
        if (h.dem) rs += h.radius[i];
    }
    o << "], \"steps\": " << a.run_steps << ", \"thermo\": " << a.thermo_every
      << ", \"n\": " << (h.size() ? h.size() : a.device_gen_n)
      << ", \"generate\": \"" << (a.device_gen ? "device" : "host") << "\", \"pos_sum\": ";
    json_vec(o, ps, 3);
    o << ", \"radius_sum\": ";
    json_num(o, rs);
    o << ", \"mass_sum\": ";
    json_num(o, ms);
    o << ", \"type_sum\": " << ts;
    o << "}";
    return o.str();
}

}  // namespace mdg_host
