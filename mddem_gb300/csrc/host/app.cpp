// app.cpp -- App, the core plugins and the device plugin.
#include "app.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <set>
#include <sstream>

#include "plugins.hpp"

namespace mdg_host {

// ---------------------------------------------------------------------------
// App
// ---------------------------------------------------------------------------
mdg_config default_config() {
    mdg_config c{};
    for (int d = 0; d < 3; d++) c.box_hi[d] = 1.0;
    c.skin_fraction = 1.0;
    c.bin_size = 1.0;
    c.check = 1;
    c.sort_every = 1000;
    c.newton = 1;
    c.lj_epsilon = 1.0;
    c.lj_sigma = 1.0;
    c.lj_cutoff = 2.5;
    c.nh_temperature = 0.85;
    c.nh_coupling = 1.0;
    c.lv_temperature = 0.85;
    c.lv_damping = 1.0;
    c.lv_seed = 12345;
    return c;
}

App::~App() {
    if (ctx) mdg_destroy(ctx);
}

App& App::add_plugin(std::unique_ptr<Plugin> p) {
    for (const std::string& r : p->requires_())
        if (std::find(provided.begin(), provided.end(), r) == provided.end())
            throw ConfigError(p->name() + " requires a plugin providing '" + r + "'");
    for (const std::string& q : p->provides()) provided.push_back(q);
    p->build(*this);
    plugins_.push_back(std::move(p));
    return *this;
}

void App::add_setup_system(Schedule set, std::function<void(App&)> f) { setup_.emplace_back(set, std::move(f)); }
void App::add_update_system(Schedule set, std::function<void(App&)> f) { update_.emplace_back(set, std::move(f)); }

void App::run_set(std::vector<std::pair<Schedule, std::function<void(App&)>>>& sys, Schedule s) {
    for (auto& e : sys)
        if (e.first == s) e.second(*this);
}

int App::start() {
    for (Schedule s : {Schedule::PreSetup, Schedule::Setup, Schedule::PostSetup}) run_set(setup_, s);
    if (opts.check || !ctx) return 0;
    // Output marks (steps into this run): every update system runs at multiples
    // of the print interval and at the last step; between marks one mdg_step
    // launch runs the whole fused schedule (InitialIntegration ...
    // PostFinalIntegration) on the device.
    step = first_step;
    std::set<long long> marks{run_steps};
    std::vector<long long> every = intervals;
    every.push_back(thermo_every);
    for (long long e : every)
        for (long long k = e; e > 0 && k < run_steps; k += e) marks.insert(k);
    run_set(update_, Schedule::LastOutput);
    for (long long k : marks) {
        if (k <= done()) continue;
        const int st = mdg_step(ctx, k - done());
        if (st != MDG_OK) {
            std::fprintf(stderr, "Error: step %lld: %s\n", step, mdg_status_string(st));
            return 2;
        }
        step = first_step + k;
        run_set(update_, Schedule::LastOutput);
    }
    for (auto& f : finish) f(*this);
    return 0;
}

// ---------------------------------------------------------------------------
// config helpers
// ---------------------------------------------------------------------------
const toml::Table* section(const App& app, const std::string& name) {
    const toml::Value* v = toml::find(app.input, name);
    if (!v) return nullptr;
    if (v->kind == toml::Value::TABLE) return v->t.get();
    // a multi-stage [[run]] uses its first stage
    if (v->kind == toml::Value::ARRAY && !v->a->empty() && v->a->front().kind == toml::Value::TABLE)
        return v->a->front().t.get();
    throw ConfigError("[" + name + "] is not a table");
}

void check_keys(const std::string& sec, const toml::Table& t, const std::set<std::string>& allowed) {
    std::string extra;
    for (const auto& kv : t)
        if (!allowed.count(kv.first)) extra += (extra.empty() ? "" : ", ") + kv.first;
    if (!extra.empty()) throw ConfigError("unknown field(s) [" + extra + "] in [" + sec + "]");
}

double num(const toml::Table* t, const std::string& key, double dflt) {
    if (!t) return dflt;
    const toml::Value* v = toml::find(*t, key);
    if (!v) return dflt;
    if (!v->is_number()) throw ConfigError("'" + key + "' must be a number");
    return v->number();
}

long long integer(const toml::Table* t, const std::string& key, long long dflt) {
    if (!t) return dflt;
    const toml::Value* v = toml::find(*t, key);
    if (!v) return dflt;
    try {
        return v->integer();
    } catch (const toml::Error&) {
        throw ConfigError("'" + key + "' must be an integer");
    }
}

bool boolean(const toml::Table* t, const std::string& key, bool dflt) {
    if (!t) return dflt;
    const toml::Value* v = toml::find(*t, key);
    if (!v) return dflt;
    if (v->kind != toml::Value::BOOL) throw ConfigError("'" + key + "' must be true or false");
    return v->b;
}

std::string text(const toml::Table* t, const std::string& key, const std::string& dflt) {
    if (!t) return dflt;
    const toml::Value* v = toml::find(*t, key);
    if (!v) return dflt;
    if (v->kind != toml::Value::STRING) throw ConfigError("'" + key + "' must be a string");
    return v->s;
}

std::vector<const toml::Table*> table_array(const toml::Table& t, const std::string& key) {
    std::vector<const toml::Table*> out;
    const toml::Value* v = toml::find(t, key);
    if (!v) return out;
    if (v->kind != toml::Value::ARRAY) throw ConfigError("'" + key + "' must be an array of tables");
    for (const toml::Value& e : *v->a) {
        if (e.kind != toml::Value::TABLE) throw ConfigError("'" + key + "' must be an array of tables");
        out.push_back(e.t.get());
    }
    return out;
}

std::vector<double> numbers(const toml::Table* t, const std::string& key) {
    std::vector<double> out;
    const toml::Value* v = t ? toml::find(*t, key) : nullptr;
    if (!v) return out;
    if (v->kind != toml::Value::ARRAY) throw ConfigError("'" + key + "' must be an array of numbers");
    for (const toml::Value& e : *v->a) {
        if (!e.is_number()) throw ConfigError("'" + key + "' must be an array of numbers");
        out.push_back(e.number());
    }
    return out;
}

// ---------------------------------------------------------------------------
// core plugins
// ---------------------------------------------------------------------------
namespace {

// InputPlugin: reads the TOML file named on the command line.
struct InputPlugin : Plugin {
    std::string name() const override { return "InputPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::PreSetup, [](App& a) {
            std::ifstream f(a.input_path);
            if (!f) throw ConfigError("cannot read " + a.input_path);
            std::stringstream ss;
            ss << f.rdbuf();
            try {
                a.input = toml::parse(ss.str());
            } catch (const toml::Error& e) {
                throw ConfigError(a.input_path + ": " + e.what());
            }
        });
    }
};

// DomainPlugin: [domain] (crates/mddem_core/src/domain.rs:46-78); periodic and
// fixed boundaries.
struct DomainPlugin : Plugin {
    std::string name() const override { return "DomainPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* d = section(a, "domain");
            if (d)
                check_keys("domain", *d,
                           {"x_low", "x_high", "y_low", "y_high", "z_low", "z_high", "x_lo", "x_hi", "y_lo", "y_hi",
                            "z_lo", "z_hi", "boundary_x", "boundary_y", "boundary_z", "shrink_wrap_padding"});
            const char* ax = "xyz";
            for (int k = 0; k < 3; k++) {
                const std::string c(1, ax[k]);
                a.cfg.box_lo[k] = num(d, c + "_low", num(d, c + "_lo", 0.0));
                a.cfg.box_hi[k] = num(d, c + "_high", num(d, c + "_hi", 1.0));
                const std::string bt = text(d, "boundary_" + c, "periodic");
                if (bt != "periodic" && bt != "fixed")
                    throw ConfigError("boundary_" + c + " = \"" + bt +
                                      "\": the GPU path supports periodic and fixed boundaries");
                a.cfg.fixed[k] = bt == "fixed" ? 1 : 0;
            }
        });
    }
};

// NeighborPlugin: [neighbor] (crates/mddem_core/src/neighbor.rs:44-80).
struct NeighborPlugin : Plugin {
    std::string name() const override { return "NeighborPlugin"; }
    std::vector<std::string> provides() const override { return {"neighbor_list"}; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* n = section(a, "neighbor");
            if (n) check_keys("neighbor", *n, {"skin_fraction", "bin_size", "every", "check", "sort_every", "newton"});
            a.cfg.skin_fraction = num(n, "skin_fraction", 1.0);
            a.cfg.bin_size = num(n, "bin_size", 1.0);
            a.cfg.every = (int)integer(n, "every", 0);
            a.cfg.check = boolean(n, "check", true) ? 1 : 0;
            a.cfg.sort_every = (int)integer(n, "sort_every", 1000);
            a.cfg.newton = boolean(n, "newton", true) ? 1 : 0;
        });
    }
};

// RunPlugin: [run] dt, steps, thermo.
struct RunPlugin : Plugin {
    std::string name() const override { return "RunPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* r = section(a, "run");
            a.cfg.dt = num(r, "dt", 0.0);
            a.run_steps = integer(r, "steps", 1000);
            a.thermo_every = integer(r, "thermo", 100);
            if (a.opts.steps >= 0) a.run_steps = a.opts.steps;
            const toml::Table* o = section(a, "output");
            a.out_dir = text(o, "dir", "output");
        });
    }
};

// PrintPlugin: the thermo line at every print interval.
struct PrintPlugin : Plugin {
    std::string name() const override { return "PrintPlugin"; }
    void build(App& app) override {
        app.add_update_system(Schedule::LastOutput, [](App& a) {
            if (!(a.thermo_every > 0 && a.done() % a.thermo_every == 0) && a.done() != a.run_steps) return;
            mdg_thermo_t t{};
            const int st = mdg_thermo(a.ctx, 0, &t);
            if (st != MDG_OK) throw ConfigError(std::string("thermo: ") + mdg_status_string(st));
            if (a.dem)
                std::printf("%10lld T_g %.6e T_rot %.6e KE %.6e |P| %.3e\n", a.step, t.granular_temp, t.rot_temp, t.ke,
                            t.momentum);
            else
                std::printf("%10lld T %.6f KE %.6e PE %.6e E %.6e P %.5f\n", a.step, t.temp, t.ke, t.pe, t.ke + t.pe,
                            t.pressure);
            std::fflush(stdout);
        });
    }
};

// The generated system's state, back on the host for the plugins that read
// it later (restart files, measurement normalisation).
void download_state(App& a) {
    const size_t n = a.device_gen_n;
    HostState& h = a.state;
    h = HostState{};
    h.dem = a.dem;
    h.tag.resize(n);
    h.type.resize(n);
    h.pos.resize(3 * n);
    h.vel.resize(3 * n);
    h.mass.resize(n);
    h.cutoff_radius.resize(n);
    mdg_state_view v{};
    v.n = n;
    v.tag = h.tag.data();
    v.type = h.type.data();
    v.pos = h.pos.data();
    v.vel = h.vel.data();
    v.mass = h.mass.data();
    v.cutoff_radius = h.cutoff_radius.data();
    if (h.dem) {
        h.radius.resize(n);
        h.inv_inertia.resize(n);
        h.omega.resize(3 * n);
        h.quat.resize(4 * n);
        h.density.assign(n, a.device_gen_density);
        v.radius = h.radius.data();
        v.inv_inertia = h.inv_inertia.data();
        v.omega = h.omega.data();
        v.quat = h.quat.data();
    }
    const int st = mdg_download_state(a.ctx, 0, &v);
    if (st != MDG_OK) throw ConfigError(std::string("mdg_download_state: ") + mdg_status_string(st));
}

// The device plugin: [gpu] settings, then (PostSetup, after the state
// plugins) the context and the upload.  It provides the systems the
// reference's NeighborPlugin, force plugins and integrators run on the host.
struct GpuPlugin : Plugin {
    std::string name() const override { return "GpuHotPathPlugin"; }
    void build(App& app) override {
        app.add_setup_system(Schedule::Setup, [](App& a) {
            const toml::Table* g = section(a, "gpu");
            if (g)
                check_keys("gpu", *g, {"precision", "rebuild_policy", "threads_per_particle", "neighbor_capacity",
                                       "history_capacity", "virial", "generate"});
            const std::string gen = text(g, "generate", "host");
            if (gen != "host" && gen != "device") throw ConfigError("generate = \"" + gen + "\": host or device");
            a.gen_device = gen == "device";
            std::string prec = text(g, "precision", "fp64");
            if (!a.opts.precision.empty()) prec = a.opts.precision;
            if (prec != "fp64" && prec != "mixed") throw ConfigError("precision = \"" + prec + "\": fp64 or mixed");
            a.cfg.precision = prec == "mixed" ? MDG_MIXED : MDG_FP64;
            const std::string pol = text(g, "rebuild_policy", "reference");
            if (pol != "reference" && pol != "displacement")
                throw ConfigError("rebuild_policy = \"" + pol + "\": reference or displacement");
            a.cfg.rebuild_policy = pol == "displacement" ? 1 : 0;
            a.cfg.threads_per_particle = (int)integer(g, "threads_per_particle", 0);
            a.cfg.neighbor_capacity = (int)integer(g, "neighbor_capacity", 0);
            a.cfg.history_capacity = (int)integer(g, "history_capacity", 0);
            a.cfg.virial = boolean(g, "virial", false) ? 1 : 0;
        });
    }
    // registered by add_core_plugins after the group plugins' PostSetup
    static void create(App& a) {
        Resumed res;
        if (a.restart_read) res = resume_from_restart(a);
        a.cfg.materials = a.materials.empty() ? nullptr : a.materials.data();
        a.cfg.n_materials = a.dem ? (int)a.materials.size() : 0;
        a.cfg.walls = a.walls.empty() ? nullptr : a.walls.data();
        a.cfg.n_walls = (int)a.walls.size();
        a.cfg.n_lj_types = a.dem ? 0 : a.lj_types;
        a.cfg.lj_pairs = a.lj_pairs.empty() ? nullptr : a.lj_pairs.data();
        if (a.opts.check) {
            if (!a.opts.write_restart.empty()) write_initial_restart(a, a.opts.write_restart);
            std::printf("%s\n", config_json(a).c_str());
            return;
        }
        if (a.device_gen && a.state.size() == 0) {  // no restart state: make the system on the device
            int st = mdg_create(&a.cfg, a.device_gen_n, &a.ctx);
            if (st != MDG_OK) throw ConfigError(std::string("mdg_create: ") + mdg_status_string(st));
            st = a.device_gen(a);
            if (st != MDG_OK) throw ConfigError(std::string("device generator: ") + mdg_status_string(st));
            download_state(a);
            std::printf("# %s N=%zu dt=%.6e steps=%lld precision=%s (generated on the device)\n", a.dem ? "dem" : "lj",
                        a.state.size(), a.cfg.dt, a.run_steps, a.cfg.precision == MDG_MIXED ? "mixed" : "fp64");
            return;
        }
        int st = mdg_create(&a.cfg, a.state.size(), &a.ctx);
        if (st != MDG_OK) throw ConfigError(std::string("mdg_create: ") + mdg_status_string(st));
        HostState& h = a.state;
        mdg_state_view v{};
        v.n = h.size();
        v.tag = h.tag.data();
        v.type = h.type.data();
        v.pos = h.pos.data();
        v.vel = h.vel.data();
        v.mass = h.mass.data();
        v.cutoff_radius = h.cutoff_radius.data();
        v.force = res.force.empty() ? nullptr : res.force.data();
        if (h.dem) {
            v.radius = h.radius.data();
            v.inv_inertia = h.inv_inertia.data();
            v.omega = h.omega.data();
            v.quat = h.quat.data();
            v.torque = res.torque.empty() ? nullptr : res.torque.data();
        }
        st = mdg_upload_state(a.ctx, 0, &v);
        if (st != MDG_OK) throw ConfigError(std::string("mdg_upload_state: ") + mdg_status_string(st));
        if (!res.hist_keys.empty()) {
            st = mdg_set_history(a.ctx, 0, res.hist_keys.size() / 2, res.hist_keys.data(), res.hist_vals.data());
            if (st != MDG_OK) throw ConfigError(std::string("mdg_set_history: ") + mdg_status_string(st));
        }
        std::printf("# %s N=%zu dt=%.6e steps=%lld precision=%s\n", a.dem ? "dem" : "lj", h.size(), a.cfg.dt,
                    a.run_steps, a.cfg.precision == MDG_MIXED ? "mixed" : "fp64");
    }
};

}  // namespace

void add_core_plugins(App& app) {
    app.add_plugin(std::make_unique<InputPlugin>());
    app.add_plugin(std::make_unique<DomainPlugin>());
    app.add_plugin(std::make_unique<NeighborPlugin>());
    app.add_plugin(std::make_unique<RunPlugin>());
    app.add_plugin(std::make_unique<PrintPlugin>());
    app.add_plugin(std::make_unique<GpuPlugin>());
    add_restart_plugin(app);
}

void add_device_context(App& app) { app.add_setup_system(Schedule::PostSetup, GpuPlugin::create); }

}  // namespace mdg_host
