// restart.hpp -- the reference's restart file (RestartData,
// crates/mddem_print/src/lib.rs:297-376) as JSON (serde_json of the struct,
// lib.rs:1062) or in bincode 1.3 form (little-endian,
// fixed-width integers, u64 length before every sequence): natoms, total_cycle,
// dt, tag, atom_type, pos/vel/force x y z, mass, cutoff_radius, the per-atom
// extension buffers (DemAtom: 17 doubles per atom in declaration order,
// dem_atom/src/lib.rs:530-557; ContactHistoryStore: per atom its contact count
// then partner tag and 7 spring values, dem_granular/src/tangential.rs:98-132),
// then the legacy rotational fields, written empty.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "app.hpp"

namespace mdg_host {

struct RestartInput {
    const HostState* state = nullptr;
    const std::vector<double>* force = nullptr;    // 3n, or null = zeros
    const std::vector<double>* torque = nullptr;   // 3n (DEM), or null = zeros
    const std::vector<double>* density = nullptr;  // n (DEM), or null = mass / (4/3 pi r^3)
    // contact history (DEM): (owner tag, partner tag) and 7 doubles each
    const std::vector<uint32_t>* hist_keys = nullptr;
    const std::vector<double>* hist_vals = nullptr;
    uint64_t step = 0;
    double dt = 0.0;
};

// The file's bytes; throws ConfigError on inconsistent sizes.
std::string restart_bincode(const RestartInput& in);
std::string restart_json(const RestartInput& in);
// restart_{step}_rank{rank}.bin (.json)
std::string restart_filename(uint64_t step, int rank = 0, bool json = false);

// A restart file read back: the state (DEM when it carries the DemAtom
// buffer), forces, torques, contact history, step and dt.
struct RestartRead {
    HostState state;
    std::vector<double> force, torque;
    std::vector<uint32_t> hist_keys;
    std::vector<double> hist_vals;
    uint64_t step = 0;
    double dt = 0.0;
};
// Parse bincode / JSON RestartData; throws ConfigError on malformed input.
RestartRead restart_read(const std::string& bytes);
RestartRead restart_read_json(const std::string& text);
// The restart file with the highest step for rank 0 and the format in `dir`,
// or "" (read_restart's scan, crates/mddem_print/src/lib.rs:1163-1185).
std::string latest_restart(const std::string& dir, bool json = false);

}  // namespace mdg_host
