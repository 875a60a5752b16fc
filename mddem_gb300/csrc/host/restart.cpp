// restart.cpp -- bincode writer and reader of the reference's RestartData.
#include "restart.hpp"

#include <cmath>
#include <cstring>
#include <filesystem>
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

// little-endian reader over the file's bytes; bounds-checked
struct Reader {
    const std::string& b;
    size_t off = 0;
    template <class T>
    T get() {
        if (off + sizeof(T) > b.size()) throw ConfigError("restart: truncated file");
        unsigned char c[sizeof(T)];
        const uint16_t probe = 1;
        unsigned char first;
        std::memcpy(&first, &probe, 1);
        for (size_t k = 0; k < sizeof(T); k++) c[k] = (unsigned char)b[off + (first == 1 ? k : sizeof(T) - 1 - k)];
        off += sizeof(T);
        T v;
        std::memcpy(&v, c, sizeof(T));
        return v;
    }
    template <class T>
    std::vector<T> seq(uint64_t width = 1) {
        const uint64_t m = get<uint64_t>();
        if (m > (b.size() - off) / (sizeof(T) * width)) throw ConfigError("restart: sequence longer than the file");
        std::vector<T> v((size_t)(m * width));
        for (auto& x : v) x = get<T>();
        return v;
    }
};

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

RestartRead restart_read(const std::string& bytes) {
    Reader r{bytes};
    RestartRead out;
    r.get<uint64_t>();  // natoms
    out.step = r.get<uint64_t>();
    out.dt = r.get<double>();
    HostState& h = out.state;
    h.tag = r.seq<uint32_t>();
    h.type = r.seq<uint32_t>();
    const size_t n = h.tag.size();
    if (h.type.size() != n) throw ConfigError("restart: tag and type lengths differ");
    std::vector<double> cols[9];
    for (auto& c : cols) {
        c = r.seq<double>();
        if (c.size() != n) throw ConfigError("restart: a vector field's length differs from natoms");
    }
    h.pos.resize(3 * n);
    h.vel.resize(3 * n);
    out.force.resize(3 * n);
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            h.pos[3 * i + d] = cols[d][i];
            h.vel[3 * i + d] = cols[3 + d][i];
            out.force[3 * i + d] = cols[6 + d][i];
        }
    h.mass = r.seq<double>();
    h.cutoff_radius = r.seq<double>();
    if (h.mass.size() != n || h.cutoff_radius.size() != n) throw ConfigError("restart: mass / cutoff_radius length");
    const uint64_t nbuf = r.get<uint64_t>();
    std::vector<std::vector<double>> bufs;
    for (uint64_t k = 0; k < nbuf; k++) bufs.push_back(r.seq<double>());
    for (int k = 0; k < 9; k++) r.seq<double>();  // legacy rotational fields
    r.seq<double>(4);                              // legacy quaternion
    if (r.off != bytes.size()) throw ConfigError("restart: trailing bytes");
    h.dem = !bufs.empty() && bufs[0].size() == (size_t)kDemPack * n;
    if (h.dem) {
        const std::vector<double>& d = bufs[0];
        h.radius.resize(n);
        h.density.resize(n);
        h.inv_inertia.resize(n);
        h.quat.resize(4 * n);
        h.omega.resize(3 * n);
        out.torque.resize(3 * n);
        for (size_t i = 0; i < n; i++) {
            const double* p = &d[(size_t)kDemPack * i];
            h.radius[i] = p[0];
            h.density[i] = p[1];
            h.inv_inertia[i] = p[2];
            for (int q = 0; q < 4; q++) h.quat[4 * i + q] = p[3 + q];
            for (int q = 0; q < 3; q++) h.omega[3 * i + q] = p[7 + q];
            for (int q = 0; q < 3; q++) out.torque[3 * i + q] = p[13 + q];
        }
        if (bufs.size() > 1) {
            const std::vector<double>& hb = bufs[1];
            size_t pos = 0;
            for (size_t i = 0; i < n; i++) {
                if (pos >= hb.size()) throw ConfigError("restart: contact-history buffer too short");
                const size_t cnt = (size_t)hb[pos++];
                for (size_t c = 0; c < cnt; c++) {
                    if (pos + 8 > hb.size()) throw ConfigError("restart: contact-history buffer too short");
                    out.hist_keys.push_back(h.tag[i]);
                    out.hist_keys.push_back((uint32_t)hb[pos]);
                    for (int q = 0; q < 7; q++) out.hist_vals.push_back(hb[pos + 1 + q]);
                    pos += 8;
                }
            }
            if (pos != hb.size()) throw ConfigError("restart: contact-history buffer length does not match its counts");
        }
    }
    return out;
}

std::string latest_restart(const std::string& dir) {
    namespace fs = std::filesystem;
    std::error_code ec;
    if (!fs::is_directory(dir, ec)) return "";
    const std::string pre = "restart_", suf = "_rank0.bin";
    long long best = -1;
    std::string name;
    for (const auto& e : fs::directory_iterator(dir, ec)) {
        const std::string f = e.path().filename().string();
        if (f.size() <= pre.size() + suf.size() || f.compare(0, pre.size(), pre) != 0 ||
            f.compare(f.size() - suf.size(), suf.size(), suf) != 0)
            continue;
        const std::string mid = f.substr(pre.size(), f.size() - pre.size() - suf.size());
        if (mid.empty() || mid.find_first_not_of("0123456789") != std::string::npos) continue;
        const long long s = std::stoll(mid);
        if (s > best) {
            best = s;
            name = f;
        }
    }
    return best < 0 ? "" : dir + "/" + name;
}

}  // namespace mdg_host
