// restart.cpp -- the reference's RestartData: bincode and JSON writers and
// readers over one field set.
#include "restart.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <map>
#include <type_traits>

namespace mdg_host {
namespace {

constexpr int kDemPack = 17;
constexpr double kPi = 3.141592653589793;
const char* const kCols[9] = {"pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "force_x", "force_y", "force_z"};
const char* const kLegacy[9] = {"omega_x", "omega_y", "omega_z", "torque_x", "torque_y",
                                "torque_z", "ang_mom_x", "ang_mom_y", "ang_mom_z"};

// RestartData's fields in declaration order (crates/mddem_print/src/lib.rs:
// 297-337); the legacy rotational fields are written empty and ignored on read.
struct Fields {
    uint64_t natoms = 0, total_cycle = 0;
    double dt = 0.0;
    std::vector<uint32_t> tag, type;
    std::vector<double> col[9];  // pos, vel, force x y z
    std::vector<double> mass, cutr;
    std::vector<std::vector<double>> bufs;
};

std::vector<double> column(const std::vector<double>* a, size_t n, int stride, int c) {
    std::vector<double> out(n, 0.0);
    if (a)
        for (size_t i = 0; i < n; i++) out[i] = (*a)[(size_t)stride * i + c];
    return out;
}

Fields to_fields(const RestartInput& in) {
    const HostState& h = *in.state;
    const size_t n = h.size();
    if (h.pos.size() != 3 * n || h.vel.size() != 3 * n || h.mass.size() != n || h.cutoff_radius.size() != n ||
        (in.force && in.force->size() != 3 * n))
        throw ConfigError("restart: inconsistent state sizes");
    Fields f;
    f.natoms = n;
    f.total_cycle = in.step;
    f.dt = in.dt;
    f.tag = h.tag;
    f.type = h.type;
    for (int c = 0; c < 3; c++) {
        f.col[c] = column(&h.pos, n, 3, c);
        f.col[3 + c] = column(&h.vel, n, 3, c);
        f.col[6 + c] = column(in.force, n, 3, c);
    }
    f.mass = h.mass;
    f.cutr = h.cutoff_radius;
    if (!h.dem) return f;
    // DemAtom, 17 doubles per atom in declaration order (dem_atom/src/lib.rs:530-557)
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
    f.bufs.push_back(std::move(dem));
    // ContactHistoryStore (tangential.rs:98-132): per atom in the file's order
    // its contact count, then partner tag and 7 spring values per contact
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
    f.bufs.push_back(std::move(hist));
    return f;
}

RestartRead from_fields(Fields&& f) {
    RestartRead out;
    out.step = f.total_cycle;
    out.dt = f.dt;
    HostState& h = out.state;
    h.tag = std::move(f.tag);
    h.type = std::move(f.type);
    const size_t n = h.tag.size();
    if (h.type.size() != n) throw ConfigError("restart: tag and type lengths differ");
    for (auto& c : f.col)
        if (c.size() != n) throw ConfigError("restart: a vector field's length differs from natoms");
    h.pos.resize(3 * n);
    h.vel.resize(3 * n);
    out.force.resize(3 * n);
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            h.pos[3 * i + d] = f.col[d][i];
            h.vel[3 * i + d] = f.col[3 + d][i];
            out.force[3 * i + d] = f.col[6 + d][i];
        }
    h.mass = std::move(f.mass);
    h.cutoff_radius = std::move(f.cutr);
    if (h.mass.size() != n || h.cutoff_radius.size() != n) throw ConfigError("restart: mass / cutoff_radius length");
    const auto& bufs = f.bufs;
    h.dem = !bufs.empty() && bufs[0].size() == (size_t)kDemPack * n;
    if (!h.dem) return out;
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
            // the count is stored as a double: it must be a whole number >= 0
            // whose entries (8 doubles each) fit in what is left of the buffer
            const double craw = hb[pos++];
            const size_t left = (hb.size() - pos) / 8;
            if (!std::isfinite(craw) || craw < 0.0 || craw != std::floor(craw) || craw > (double)left)
                throw ConfigError("restart: contact-history count is not a whole number within the buffer");
            const size_t cnt = (size_t)craw;
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
    return out;
}

// ---- bincode 1.3: little-endian, fixed-width integers, u64 length before
// every sequence
bool little_endian() {
    const uint16_t probe = 1;
    unsigned char first;
    std::memcpy(&first, &probe, 1);
    return first == 1;
}

template <class T>
void put(std::string& out, T v) {
    unsigned char b[sizeof(T)];
    std::memcpy(b, &v, sizeof(T));
    if (little_endian()) {
        out.append(reinterpret_cast<const char*>(b), sizeof(T));
    } else {
        for (size_t k = sizeof(T); k-- > 0;) out.push_back((char)b[k]);
    }
}

template <class T>
void put_seq(std::string& out, const std::vector<T>& v) {
    put<uint64_t>(out, (uint64_t)v.size());
    for (const T& x : v) put<T>(out, x);
}

std::string encode_bincode(const Fields& f) {
    std::string out;
    put<uint64_t>(out, f.natoms);
    put<uint64_t>(out, f.total_cycle);
    put<double>(out, f.dt);
    put_seq(out, f.tag);
    put_seq(out, f.type);
    for (const auto& c : f.col) put_seq(out, c);
    put_seq(out, f.mass);
    put_seq(out, f.cutr);
    put<uint64_t>(out, (uint64_t)f.bufs.size());
    for (const auto& b : f.bufs) put_seq(out, b);
    for (int k = 0; k < 9; k++) put<uint64_t>(out, 0);  // omega, torque, ang_mom x y z: empty
    put<uint64_t>(out, 0);                               // quaternion: empty
    return out;
}

// bounds-checked little-endian reader over the file's bytes
struct Reader {
    const std::string& b;
    size_t off = 0;
    template <class T>
    T get() {
        if (off + sizeof(T) > b.size()) throw ConfigError("restart: truncated file");
        unsigned char c[sizeof(T)];
        const bool le = little_endian();
        for (size_t k = 0; k < sizeof(T); k++) c[k] = (unsigned char)b[off + (le ? k : sizeof(T) - 1 - k)];
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

Fields decode_bincode(const std::string& bytes) {
    Reader r{bytes};
    Fields f;
    f.natoms = r.get<uint64_t>();
    f.total_cycle = r.get<uint64_t>();
    f.dt = r.get<double>();
    f.tag = r.seq<uint32_t>();
    f.type = r.seq<uint32_t>();
    for (auto& c : f.col) c = r.seq<double>();
    f.mass = r.seq<double>();
    f.cutr = r.seq<double>();
    const uint64_t nbuf = r.get<uint64_t>();
    if (nbuf > bytes.size()) throw ConfigError("restart: buffer count longer than the file");
    for (uint64_t k = 0; k < nbuf; k++) f.bufs.push_back(r.seq<double>());
    for (int k = 0; k < 9; k++) r.seq<double>();  // legacy rotational fields
    r.seq<double>(4);                              // legacy quaternion
    if (r.off != bytes.size()) throw ConfigError("restart: trailing bytes");
    return f;
}

// ---- JSON (serde_json of the same struct, lib.rs:1062): one object with the
// fields in declaration order; numbers printed with 17 significant digits
// so they read back exactly
void json_num(std::string& out, double x) {
    if (!std::isfinite(x)) {
        out += "null";  // serde_json's form of a non-finite f64
        return;
    }
    char b[40];
    std::snprintf(b, sizeof(b), "%.17g", x);
    out += b;
}

template <class T>
void json_arr(std::string& out, const std::vector<T>& v) {
    out += '[';
    for (size_t k = 0; k < v.size(); k++) {
        if (k) out += ',';
        if constexpr (std::is_integral<T>::value)
            out += std::to_string(v[k]);
        else
            json_num(out, v[k]);
    }
    out += ']';
}

std::string encode_json(const Fields& f) {
    std::string out = "{\"natoms\":" + std::to_string(f.natoms) + ",\"total_cycle\":" + std::to_string(f.total_cycle) +
                      ",\"dt\":";
    json_num(out, f.dt);
    out += ",\"tag\":";
    json_arr(out, f.tag);
    out += ",\"atom_type\":";
    json_arr(out, f.type);
    for (int c = 0; c < 9; c++) {
        out += ",\"" + std::string(kCols[c]) + "\":";
        json_arr(out, f.col[c]);
    }
    out += ",\"mass\":";
    json_arr(out, f.mass);
    out += ",\"cutoff_radius\":";
    json_arr(out, f.cutr);
    out += ",\"atom_data_buffers\":[";
    for (size_t k = 0; k < f.bufs.size(); k++) {
        if (k) out += ',';
        json_arr(out, f.bufs[k]);
    }
    out += ']';
    for (const char* name : kLegacy) out += ",\"" + std::string(name) + "\":[]";
    out += ",\"quaternion\":[]}";
    return out;
}

// A JSON value of the restart object: numbers, arrays (nested) and the top
// object; strings and booleans do not occur in RestartData.
struct JVal {
    enum Kind { NUM, ARR, OBJ, NUL } kind = NUL;
    double num = 0.0;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
};

struct JParser {
    const std::string& s;
    size_t i = 0;
    void ws() {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) i++;
    }
    [[noreturn]] void fail(const char* what) {
        throw ConfigError(std::string("restart JSON: ") + what + " at offset " + std::to_string(i));
    }
    JVal value(int depth) {
        if (depth > 8) fail("nesting too deep");
        ws();
        if (i >= s.size()) fail("unexpected end");
        JVal v;
        if (s[i] == '[') {
            v.kind = JVal::ARR;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') {
                i++;
                return v;
            }
            for (;;) {
                v.arr.push_back(value(depth + 1));
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                } else if (i < s.size() && s[i] == ']') {
                    i++;
                    return v;
                } else {
                    fail("expected , or ]");
                }
            }
        }
        if (s[i] == '{') {
            v.kind = JVal::OBJ;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') {
                i++;
                return v;
            }
            for (;;) {
                ws();
                if (i >= s.size() || s[i] != '"') fail("expected a key");
                const size_t e = s.find('"', i + 1);
                if (e == std::string::npos) fail("unterminated key");
                std::string key = s.substr(i + 1, e - i - 1);
                i = e + 1;
                ws();
                if (i >= s.size() || s[i] != ':') fail("expected :");
                i++;
                v.obj.emplace_back(std::move(key), value(depth + 1));
                ws();
                if (i < s.size() && s[i] == ',') {
                    i++;
                } else if (i < s.size() && s[i] == '}') {
                    i++;
                    return v;
                } else {
                    fail("expected , or }");
                }
            }
        }
        if (s.compare(i, 4, "null") == 0) {
            i += 4;
            v.kind = JVal::NUL;
            v.num = NAN;
            return v;
        }
        const char* p = s.c_str() + i;
        char* end = nullptr;
        v.num = std::strtod(p, &end);
        if (end == p) fail("expected a number");
        i += (size_t)(end - p);
        v.kind = JVal::NUM;
        return v;
    }
};

const JVal* member(const JVal& o, const char* key) {
    for (const auto& kv : o.obj)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

std::vector<double> doubles(const JVal* v, const char* key) {
    std::vector<double> out;
    if (!v) throw ConfigError(std::string("restart JSON: missing ") + key);
    if (v->kind != JVal::ARR) throw ConfigError(std::string("restart JSON: ") + key + " is not an array");
    for (const JVal& e : v->arr) {
        if (e.kind != JVal::NUM && e.kind != JVal::NUL)
            throw ConfigError(std::string("restart JSON: ") + key + " holds a non-number");
        out.push_back(e.num);
    }
    return out;
}

std::vector<uint32_t> u32s(const JVal* v, const char* key) {
    std::vector<uint32_t> out;
    for (double x : doubles(v, key)) {
        if (!(x >= 0.0 && x <= 4294967295.0 && x == std::floor(x)))
            throw ConfigError(std::string("restart JSON: ") + key + " holds a non-u32");
        out.push_back((uint32_t)x);
    }
    return out;
}

Fields decode_json(const std::string& text) {
    JParser p{text};
    const JVal root = p.value(0);
    p.ws();
    if (p.i != text.size()) p.fail("trailing characters");
    if (root.kind != JVal::OBJ) throw ConfigError("restart JSON: not an object");
    auto scalar = [&](const char* key) {
        const JVal* v = member(root, key);
        if (!v || v->kind != JVal::NUM) throw ConfigError(std::string("restart JSON: missing ") + key);
        return v->num;
    };
    Fields f;
    f.natoms = (uint64_t)scalar("natoms");
    f.total_cycle = (uint64_t)scalar("total_cycle");
    f.dt = scalar("dt");
    f.tag = u32s(member(root, "tag"), "tag");
    f.type = u32s(member(root, "atom_type"), "atom_type");
    for (int c = 0; c < 9; c++) f.col[c] = doubles(member(root, kCols[c]), kCols[c]);
    f.mass = doubles(member(root, "mass"), "mass");
    f.cutr = doubles(member(root, "cutoff_radius"), "cutoff_radius");
    const JVal* b = member(root, "atom_data_buffers");
    if (!b || b->kind != JVal::ARR) throw ConfigError("restart JSON: missing atom_data_buffers");
    for (const JVal& e : b->arr) f.bufs.push_back(doubles(&e, "atom_data_buffers"));
    return f;
}

}  // namespace

std::string restart_filename(uint64_t step, int rank, bool json) {
    return "restart_" + std::to_string(step) + "_rank" + std::to_string(rank) + (json ? ".json" : ".bin");
}

std::string restart_bincode(const RestartInput& in) { return encode_bincode(to_fields(in)); }
std::string restart_json(const RestartInput& in) { return encode_json(to_fields(in)); }
RestartRead restart_read(const std::string& bytes) { return from_fields(decode_bincode(bytes)); }
RestartRead restart_read_json(const std::string& text) { return from_fields(decode_json(text)); }

std::string latest_restart(const std::string& dir, bool json) {
    namespace fs = std::filesystem;
    std::error_code ec;
    if (!fs::is_directory(dir, ec)) return "";
    const std::string pre = "restart_", suf = json ? "_rank0.json" : "_rank0.bin";
    long long best = -1;
    std::string name;
    for (const auto& e : fs::directory_iterator(dir, ec)) {
        const std::string f = e.path().filename().string();
        if (f.size() <= pre.size() + suf.size() || f.compare(0, pre.size(), pre) != 0 ||
            f.compare(f.size() - suf.size(), suf.size(), suf) != 0)
            continue;
        const std::string mid = f.substr(pre.size(), f.size() - pre.size() - suf.size());
        if (mid.empty() || mid.size() > 18 || mid.find_first_not_of("0123456789") != std::string::npos) continue;
        const long long s = std::stoll(mid);
        if (s > best) {
            best = s;
            name = f;
        }
    }
    return best < 0 ? "" : dir + "/" + name;
}

}  // namespace mdg_host
