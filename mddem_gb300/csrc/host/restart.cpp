// restart.cpp -- bincode writer of the reference's RestartData.
#include "restart.hpp"

#include <cmath>
#include <cstring>
#include <map>

namespace mdg_host {
namespace {

constexpr int kDemPack = 17;
constexpr double kPi = 3.141592653589793;

// little-endian byte order of the bincode encoding
template <class T>
void put(std::string& out, T v) {
    unsigned char b[sizeof(T)];
    std::memcpy(b, &v, sizeof(T));
    const uint16_t probe = 1;
    unsigned char first;
    std::memcpy(&first, &probe, 1);
    if (first == 1) {
        out.append(reinterpret_cast<const char*>(b), sizeof(T));
    } else {
        for (size_t k = sizeof(T); k-- > 0;) out.push_back((char)b[k]);
    }
}

template <class T>
void seq(std::string& out, const std::vector<T>& v) {
    put<uint64_t>(out, (uint64_t)v.size());
    for (const T& x : v) put<T>(out, x);
}

std::vector<double> column(const std::vector<double>* a, size_t n, int stride, int c) {
    std::vector<double> out(n, 0.0);
    if (a)
        for (size_t i = 0; i < n; i++) out[i] = (*a)[(size_t)stride * i + c];
    return out;
}

}  // namespace

std::string restart_filename(uint64_t step, int rank) {
    return "restart_" + std::to_string(step) + "_rank" + std::to_string(rank) + ".bin";
}

std::string restart_bincode(const RestartInput& in) {
    const HostState& h = *in.state;
    const size_t n = h.size();
    if (h.pos.size() != 3 * n || h.vel.size() != 3 * n || h.mass.size() != n || h.cutoff_radius.size() != n ||
        (in.force && in.force->size() != 3 * n))
        throw ConfigError("restart: inconsistent state sizes");
    std::string out;
    put<uint64_t>(out, (uint64_t)n);
    put<uint64_t>(out, in.step);
    put<double>(out, in.dt);
    seq(out, h.tag);
    seq(out, h.type);
    for (int c = 0; c < 3; c++) seq(out, column(&h.pos, n, 3, c));
    for (int c = 0; c < 3; c++) seq(out, column(&h.vel, n, 3, c));
    for (int c = 0; c < 3; c++) seq(out, column(in.force, n, 3, c));
    seq(out, h.mass);
    seq(out, h.cutoff_radius);
    if (h.dem) {
        put<uint64_t>(out, 2);
        std::vector<double> dem((size_t)kDemPack * n, 0.0);
        for (size_t i = 0; i < n; i++) {
            double* d = &dem[(size_t)kDemPack * i];
            const double r = h.radius[i];
            d[0] = r;
            d[1] = in.density ? (*in.density)[i] : h.mass[i] / (4.0 / 3.0 * kPi * std::pow(r, 3.0));
            d[2] = h.inv_inertia[i];
            for (int q = 0; q < 4; q++) d[3 + q] = h.quat[4 * i + q];
            for (int q = 0; q < 3; q++) d[7 + q] = h.omega[3 * i + q];
            // ang_mom (10..12) and body_id (16) stay 0
            for (int q = 0; q < 3; q++) d[13 + q] = in.torque ? (*in.torque)[3 * i + q] : 0.0;
        }
        seq(out, dem);
        // contact history grouped under each atom in the file's atom order
        std::map<uint32_t, std::vector<size_t>> per;
        const size_t nh = in.hist_keys ? in.hist_keys->size() / 2 : 0;
        if (in.hist_keys && (!in.hist_vals || in.hist_vals->size() != 7 * nh))
            throw ConfigError("restart: history keys and values differ in length");
        for (size_t e = 0; e < nh; e++) per[(*in.hist_keys)[2 * e]].push_back(e);
        std::vector<double> hist;
        for (size_t i = 0; i < n; i++) {
            auto it = per.find(h.tag[i]);
            if (it == per.end()) {
                hist.push_back(0.0);
                continue;
            }
            hist.push_back((double)it->second.size());
            for (size_t e : it->second) {
                hist.push_back((double)(*in.hist_keys)[2 * e + 1]);
                for (int q = 0; q < 7; q++) hist.push_back((*in.hist_vals)[7 * e + q]);
            }
        }
        seq(out, hist);
    } else {
        put<uint64_t>(out, 0);
    }
    for (int k = 0; k < 9; k++) put<uint64_t>(out, 0);  // omega, torque, ang_mom x y z: empty
    put<uint64_t>(out, 0);                               // quaternion: empty
    return out;
}

}  // namespace mdg_host
