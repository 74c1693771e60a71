// namelist.hpp -- reader for the Fortran namelist groups the reference drivers
// take on standard input (&MCDATA in pimd_par.f90:42-45, &RPIDATA in
// rpi_ser.f90:22-24) and for the plain-text data files they open
// (masses.dat, well1.dat, well2.dat, path.xyz).
#pragma once
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace pgdrv {

inline std::string lower(std::string s) {
    for (auto &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

// Key -> raw value text (lower-case keys, quotes stripped from strings).
// Like a Fortran namelist read, a run stops on a key the program does not take
// or a value that does not convert: the accessors record the keys they are
// asked for and the values that fail, and check() reports both.
class Namelist {
  public:
    std::map<std::string, std::string> kv;
    mutable std::set<std::string> used;
    mutable std::vector<std::string> errors;

    // Parses the first group named `group` ("&group ... /") from text.
    static Namelist parse(const std::string &text, const std::string &group) {
        Namelist nl;
        std::string t = text;
        std::string low = lower(t);
        size_t p = low.find("&" + lower(group));
        if (p == std::string::npos) throw std::runtime_error("namelist group &" + group + " not found");
        p += group.size() + 1;
        // body ends at an unquoted '/' or '&end'
        std::string body;
        bool inq = false;
        char q = 0;
        for (size_t i = p; i < t.size(); i++) {
            char c = t[i];
            if (inq) {
                if (c == q) inq = false;
                body += c;
                continue;
            }
            if (c == '\'' || c == '"') {
                inq = true;
                q = c;
                body += c;
                continue;
            }
            if (c == '/') break;
            if (c == '&' && lower(t.substr(i, 4)) == "&end") break;
            if (c == '!') {  // comment to end of line
                while (i < t.size() && t[i] != '\n') i++;
                body += ' ';
                continue;
            }
            body += c;
        }
        // split into key = value pairs at top-level commas / whitespace before "key ="
        size_t i = 0;
        auto skip = [&]() {
            while (i < body.size() && (std::isspace((unsigned char)body[i]) || body[i] == ',')) i++;
        };
        while (true) {
            skip();
            if (i >= body.size()) break;
            size_t ks = i;
            while (i < body.size() && body[i] != '=' && !std::isspace((unsigned char)body[i])) i++;
            std::string key = lower(body.substr(ks, i - ks));
            while (i < body.size() && std::isspace((unsigned char)body[i])) i++;
            if (i >= body.size() || body[i] != '=') throw std::runtime_error("namelist: expected '=' after " + key);
            i++;
            while (i < body.size() && std::isspace((unsigned char)body[i])) i++;
            std::string val;
            if (i < body.size() && (body[i] == '\'' || body[i] == '"')) {
                char qq = body[i++];
                while (i < body.size() && body[i] != qq) val += body[i++];
                i++;
            } else {
                while (i < body.size() && body[i] != ',' && !std::isspace((unsigned char)body[i])) val += body[i++];
            }
            nl.kv[key] = val;
        }
        return nl;
    }

    bool has(const std::string &k) const { return kv.count(lower(k)) > 0; }

    double real(const std::string &k, double def) const {
        auto it = find(k);
        if (it == kv.end()) return def;
        std::string v = it->second;
        for (auto &c : v)
            if (c == 'd' || c == 'D') c = 'e';  // Fortran double exponent
        char *end = nullptr;
        const double x = std::strtod(v.c_str(), &end);
        if (v.empty() || end != v.c_str() + v.size()) {
            errors.push_back("namelist: " + lower(k) + " = '" + it->second + "' is not a number");
            return def;
        }
        return x;
    }
    long long integer(const std::string &k, long long def) const {
        auto it = find(k);
        if (it == kv.end()) return def;
        return (long long)real(k, (double)def);  // accepts 5e6-style integers
    }
    bool logical(const std::string &k, bool def) const {
        auto it = find(k);
        if (it == kv.end()) return def;
        std::string v = lower(it->second);
        if (v.size() && v[0] == '.') v = v.substr(1);
        if (v.empty() || (v[0] != 't' && v[0] != 'f')) {
            errors.push_back("namelist: " + lower(k) + " = '" + it->second + "' is not a logical");
            return def;
        }
        return v[0] == 't';
    }
    std::string str(const std::string &k, const std::string &def) const {
        auto it = find(k);
        return it == kv.end() ? def : it->second;
    }
    // Reference keys that have no effect in this program.
    void accept(std::initializer_list<const char *> keys) const {
        for (const char *k : keys) used.insert(lower(k));
    }
    // Reports unknown keys and unconvertible values on err; false if any.
    bool check(std::ostream &err) const {
        bool ok = errors.empty();
        for (const auto &e : errors) err << e << "\n";
        for (const auto &p : kv)
            if (!used.count(p.first)) {
                err << "namelist: unknown key '" << p.first << "'\n";
                ok = false;
            }
        return ok;
    }

  private:
    std::map<std::string, std::string>::const_iterator find(const std::string &k) const {
        used.insert(lower(k));
        return kv.find(lower(k));
    }
};

// Range checks of namelist values: each failed condition prints "namelist:
// <what>" on err; returns false if any failed.
struct RangeCheck {
    std::ostream &err;
    bool ok = true;
    void need(bool cond, const char *what) {
        if (!cond) {
            err << "namelist: " << what << "\n";
            ok = false;
        }
    }
};

inline std::string read_all(std::istream &in) {
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

// masses.dat: "label mass" per atom (pimd_par.f90:154-158).
inline void read_masses(const std::string &path, int natom, std::vector<std::string> &label,
                        std::vector<double> &mass) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    label.resize(natom);
    mass.resize(natom);
    for (int j = 0; j < natom; j++)
        if (!(f >> label[j] >> mass[j])) throw std::runtime_error("short masses file " + path);
}

// well*.dat: ndim coordinates per atom (pimd_par.f90:123-130), stored as x[atom*ndim + dim].
inline std::vector<double> read_well(const std::string &path, int ndim, int natom, int xunit) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<double> w((size_t)ndim * natom);
    for (auto &v : w)
        if (!(f >> v)) throw std::runtime_error("short well file " + path);
    if (xunit == 2)
        for (auto &v : w) v /= 0.529177;  // Angstrom -> bohr (pimd_par.f90:133-136)
    return w;
}

// path.xyz: npath frames of "natom / comment / label x y z" (instantonmod.f90:916-935).
inline std::vector<std::vector<double>> read_path_xyz(const std::string &path, int npath, int ndim, int natom,
                                                      int xunit) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<std::vector<double>> frames;
    std::string line;
    for (int i = 0; i < npath; i++) {
        if (!std::getline(f, line)) throw std::runtime_error("short path file");
        if (!std::getline(f, line)) throw std::runtime_error("short path file");
        std::vector<double> fr((size_t)ndim * natom);
        for (int j = 0; j < natom; j++) {
            if (!std::getline(f, line)) throw std::runtime_error("short path file");
            std::istringstream ls(line);
            std::string lab;
            ls >> lab;
            for (int k = 0; k < ndim; k++) ls >> fr[(size_t)j * ndim + k];
        }
        if (xunit == 2)
            for (auto &v : fr) v /= 0.529177;
        frames.push_back(fr);
    }
    return frames;
}

// Frames as xyz in Angstrom (bohr * 0.529177), each "natom / comment /
// label x y z" (the aligned_wells.xyz / aligned_ends.xyz layout,
// pimd_par.f90:170-183, rpi_ser.f90:81-92).  Frames are x[atom*ndim + dim].
inline bool write_xyz(const std::string &path, const std::vector<std::vector<double>> &frames,
                      const std::vector<std::string> &comments, int ndim, int natom,
                      const std::vector<std::string> &label) {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    for (size_t i = 0; i < frames.size(); i++) {
        std::fprintf(f, " %d\n %s\n", natom, i < comments.size() ? comments[i].c_str() : "");
        for (int j = 0; j < natom; j++) {
            std::fprintf(f, " %s", j < (int)label.size() ? label[j].c_str() : "X");
            for (int d = 0; d < ndim; d++) std::fprintf(f, " %.17g", frames[i][(size_t)j * ndim + d] * 0.529177);
            std::fprintf(f, "\n");
        }
    }
    return std::fclose(f) == 0;
}

// The side files read_path leaves (instantonmod.f90:1013-1031): testspline.csv
// with "dim atom y2(1..npath)" per coordinate (dimension outer, atom inner) for
// the path's spline second derivatives y2[dof], dof = atom*ndim + dim; and
// aligned.xyz with the n start beads xt[dof*n + bead] in Angstrom under the
// rotation angles of the path's alignment.
inline bool write_read_path_files(const std::vector<std::vector<double>> &y2, const std::vector<double> &xt,
                                  int64_t n, int ndim, int natom, const std::vector<std::string> &label,
                                  const double angles[3]) {
    FILE *f = std::fopen("testspline.csv", "w");
    if (!f) return false;
    for (int d = 0; d < ndim; d++)
        for (int j = 0; j < natom; j++) {
            std::fprintf(f, " %d %d", d + 1, j + 1);
            for (double v : y2[(size_t)j * ndim + d]) std::fprintf(f, " %.17g", v);
            std::fprintf(f, "\n");
        }
    if (std::fclose(f) != 0) return false;
    f = std::fopen("aligned.xyz", "w");
    if (!f) return false;
    for (int64_t b = 0; b < n; b++) {
        std::fprintf(f, " %d\n rotation angles: %.17g %.17g %.17g\n", natom, angles[0], angles[1], angles[2]);
        for (int j = 0; j < natom; j++) {
            std::fprintf(f, " %s", j < (int)label.size() ? label[j].c_str() : "X");
            for (int d = 0; d < ndim; d++) std::fprintf(f, " %.17g", xt[(size_t)(j * ndim + d) * n + b] * 0.529177);
            std::fprintf(f, "\n");
        }
    }
    return std::fclose(f) == 0;
}

// {"well1": [...], "well2": [...], "path": [[...], ...]} on standard output
// (bohr, x[atom*ndim + dim]): the start configurations a driver run would use.
inline void print_frames_json(const std::vector<double> &w1, const std::vector<double> &w2,
                              const std::vector<std::vector<double>> &frames) {
    auto arr = [](const std::vector<double> &v) {
        std::printf("[");
        for (size_t k = 0; k < v.size(); k++) std::printf("%s%.17g", k ? ", " : "", v[k]);
        std::printf("]");
    };
    std::printf("{\"well1\": ");
    arr(w1);
    std::printf(", \"well2\": ");
    arr(w2);
    std::printf(", \"path\": [");
    for (size_t i = 0; i < frames.size(); i++) {
        if (i) std::printf(", ");
        arr(frames[i]);
    }
    std::printf("]}\n");
}

}  // namespace pgdrv
