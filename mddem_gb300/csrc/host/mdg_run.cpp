// mdg_run -- run a reference TOML config on the GB300 path from C++:
//
//   mdg_run config.toml [--steps N] [--seed S] [--precision fp64|mixed] [--check]
//                       [--write-restart PATH]
//
// The reference's examples compose `CorePlugins` with `GranularDefaultPlugins`
// or `LJDefaultPlugins` (examples/*/main.rs); this does the same from the
// config: [lj] or [lattice] selects the LJ group, otherwise the granular
// group, plus WallPlugin for [[wall]] and LangevinPlugin for [langevin].
// --check resolves the configuration and the initial state and prints them
// as JSON without touching a device (--write-restart also writes that initial
// state as a restart file).  A configuration error prints its
// message and exits with status 1, like the reference.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>

#include "app.hpp"
#include "plugins.hpp"

using namespace mdg_host;

static int usage() {
    std::fprintf(stderr,
                 "usage: mdg_run config.toml [--steps N] [--seed S] [--precision fp64|mixed] [--check] "
                 "[--write-restart PATH]\n");
    return 1;
}

int main(int argc, char** argv) {
    App app;
    std::string path;
    for (int k = 1; k < argc; k++) {
        const std::string a = argv[k];
        auto next = [&](const char* what) -> const char* {
            if (k + 1 >= argc) {
                std::fprintf(stderr, "Error: %s needs a value\n", what);
                std::exit(1);
            }
            return argv[++k];
        };
        if (a == "--steps") app.opts.steps = std::atoll(next("--steps"));
        else if (a == "--seed") app.opts.seed = std::strtoull(next("--seed"), nullptr, 10);
        else if (a == "--precision") app.opts.precision = next("--precision");
        else if (a == "--check") app.opts.check = true;
        else if (a == "--write-restart") app.opts.write_restart = next("--write-restart");
        else if (a == "-h" || a == "--help") return usage();
        else if (!a.empty() && a[0] == '-') return usage();
        else path = a;
    }
    if (path.empty()) return usage();
    app.input_path = path;
    try {
        add_core_plugins(app);
        // the plugin groups depend on the config's sections, which InputPlugin
        // reads only in PreSetup: look at the document once here to choose them
        App probe;
        {
            std::FILE* f = std::fopen(path.c_str(), "rb");
            if (!f) throw ConfigError("cannot read " + path);
            std::string text;
            char buf[65536];
            size_t got;
            while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
            std::fclose(f);
            try {
                probe.input = toml::parse(text);
            } catch (const toml::Error& e) {
                throw ConfigError(path + ": " + e.what());
            }
        }
        const bool lj = toml::find(probe.input, "lj") || toml::find(probe.input, "lattice");
        if (lj) {
            add_lj_plugins(app);
        } else {
            add_granular_plugins(app);
            if (toml::find(probe.input, "wall")) add_wall_plugin(app);
        }
        if (toml::find(probe.input, "langevin")) add_langevin_plugin(app);
        add_device_context(app);
        return app.start();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "Error: %s\n", e.what());
        return 1;
    }
}
