// plugins.hpp -- helpers shared by the plugin sources.
#pragma once
#include <set>
#include <string>
#include <vector>

#include "app.hpp"

namespace mdg_host {

// The TOML table `name` (the first stage when it is an array of tables), or
// nullptr when absent.
const toml::Table* section(const App& app, const std::string& name);
// deny_unknown_fields: ConfigError naming the unknown keys.
void check_keys(const std::string& sec, const toml::Table& t, const std::set<std::string>& allowed);
double num(const toml::Table* t, const std::string& key, double dflt);
long long integer(const toml::Table* t, const std::string& key, long long dflt);
bool boolean(const toml::Table* t, const std::string& key, bool dflt);
std::string text(const toml::Table* t, const std::string& key, const std::string& dflt);
std::vector<const toml::Table*> table_array(const toml::Table& t, const std::string& key);
// A number array (absent = empty).
std::vector<double> numbers(const toml::Table* t, const std::string& key);

// The device context and the upload (PostSetup, after the state plugins).
void add_device_context(App& app);
// [restart] files (registered by the core group).
void add_restart_plugin(App& app);
// The initial state (after the state plugins) as a step-0 restart file
// (JSON when the path ends in .json, else bincode).
void write_initial_restart(const App& a, const std::string& path);

// [restart] read = true (read_restart, crates/mddem_print/src/lib.rs:1152-1251):
// the latest restart_{step}_rank0 file of the configured format in
// <output>/restart replaces the state
// and sets first_step to its step; the forces, torques and contact history it
// returns go to the device with the upload.  No file: a note, the state stays.
struct Resumed {
    std::vector<double> force, torque;
    std::vector<uint32_t> hist_keys;
    std::vector<double> hist_vals;
};
Resumed resume_from_restart(App& a);

}  // namespace mdg_host
