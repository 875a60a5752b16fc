// app.hpp -- the host side above the C ABI, shaped like the reference's
// grass App: plugins (grouped as CorePlugins, GranularDefaultPlugins,
// LJDefaultPlugins, crates/mddem/src/lib.rs:212-270 and
// crates/dem_granular/src/lib.rs:135-148) register setup systems that read
// their TOML sections into the device configuration and initial state, and
// update systems in the reference's schedule sets.  The per-step physics of
// those plugins runs on the device (one mdg_step launch advances every step
// up to the next output), so their update systems here are the output ones.
#pragma once
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/mdg.h"
#include "toml.hpp"

namespace mdg_host {

// ParticleSimScheduleSet (crates/mddem_core/src/schedule.rs:22-52) plus the
// setup sets of ScheduleSetupSet.
enum class Schedule {
    PreSetup, Setup, PostSetup,
    PreInitialIntegration, InitialIntegration, PostInitialIntegration, PreExchange, Exchange, PreNeighbor,
    Neighbor, PreForce, Force, PostForce, PreFinalIntegration, FinalIntegration, PostFinalIntegration,
    LastOutput
};

// Invalid configuration: the reference prints the message and exits with 1.
struct ConfigError : std::runtime_error {
    explicit ConfigError(const std::string& m) : std::runtime_error(m) {}
};

// Atom + DemAtom state on the host (SoA, xyz interleaved), the upload source.
struct HostState {
    bool dem = true;
    std::vector<uint32_t> tag, type;
    std::vector<double> pos, vel, mass, cutoff_radius, radius, density, inv_inertia, omega, quat;
    size_t size() const { return tag.size(); }
};

// Command-line overrides of the config.
struct Options {
    long long steps = -1;       // [run] steps unless >= 0
    uint64_t seed = 0;
    std::string precision;      // "fp64" | "mixed" | "" (config)
    bool check = false;         // resolve and print the configuration, no device
    std::string write_restart;  // with check: write the initial state as a restart file here
};

class App;

// The defaults of the config structs the plugins read (sections absent).
mdg_config default_config();

class Plugin {
public:
    virtual ~Plugin() = default;
    virtual std::string name() const = 0;
    virtual std::vector<std::string> provides() const { return {}; }
    virtual std::vector<std::string> requires_() const { return {}; }
    virtual void build(App& app) = 0;
};

class App {
public:
    App& add_plugin(std::unique_ptr<Plugin> p);
    void add_setup_system(Schedule set, std::function<void(App&)> f);
    void add_update_system(Schedule set, std::function<void(App&)> f);
    // Runs the setup sets, then the steps; returns the process exit status.
    int start();

    // resources
    std::string input_path;
    toml::Table input;              // the parsed TOML document
    Options opts;
    bool dem = true;                // granular (DEM) or LJ, from the plugin groups
    mdg_config cfg = default_config();
    std::vector<mdg_material> materials;
    std::vector<std::string> material_names;
    std::vector<mdg_wall> walls;
    int lj_types = 0;                       // [lj] types: > 1 = multi-type mode
    std::vector<mdg_lj_pair> lj_pairs;      // its n x n pair table
    HostState state;
    // [gpu] generate = "device": the state plugins leave `state` empty and
    // register the device generator of their system instead; the device
    // plugin creates the context for device_gen_n particles, runs it, and
    // downloads the generated state into `state` (densities: device_gen_density)
    bool gen_device = false;
    size_t device_gen_n = 0;
    double device_gen_density = 0.0;
    std::function<int(App&)> device_gen;
    long long run_steps = 1000, thermo_every = 100;
    std::vector<long long> intervals;   // other output intervals (measurements)
    long long step = 0;             // step counter: first_step + the steps done in this run
    long long first_step = 0;       // the restart's step when [restart] read resumed one
    bool restart_read = false;      // [restart] read = true
    bool restart_json = false;      // [restart] format = "json" (else bincode)
    long long done() const { return step - first_step; }
    mdg_ctx* ctx = nullptr;
    std::vector<std::string> provided;
    std::string out_dir = "output";
    std::vector<std::function<void(App&)>> finish;  // run after the last step

    ~App();

private:
    std::vector<std::unique_ptr<Plugin>> plugins_;
    std::vector<std::pair<Schedule, std::function<void(App&)>>> setup_, update_;
    void run_set(std::vector<std::pair<Schedule, std::function<void(App&)>>>& sys, Schedule s);
};

// Plugin groups (the reference's names and members).
void add_core_plugins(App& app);        // Input, Domain, Neighbor, Run, Print + the device plugin
void add_granular_plugins(App& app);    // DemAtom, DemAtomInsert, VelocityVerlet, HertzMindlin, Rotational, GranularTemp
void add_lj_plugins(App& app);          // Lattice, LJForce, NoseHoover, Measure
void add_wall_plugin(App& app);
void add_langevin_plugin(App& app);

// JSON of the resolved device configuration and the initial state summary.
std::string config_json(const App& app);

}  // namespace mdg_host
