// Names of the surfaces the namelist drivers accept (key pes) and the
// parameter file they read (key pes_params, one number per entry).
#pragma once
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "namelist.hpp"

namespace pgdrv {

inline int pes_id_of(const std::string &s) {
    const std::string p = lower(s);
    if (p == "1d") return PG_PES_1D;
    if (p == "2dtest") return PG_PES_2DTEST;
    if (p == "synth9") return PG_PES_SYNTH9;
    if (p == "synth18") return PG_PES_SYNTH18;
    if (p == "distgauss") return PG_PES_DISTGAUSS;
    if (p == "harmonic") return PG_PES_HARMONIC;
    throw std::runtime_error("unknown pes '" + s + "'");
}

inline std::vector<double> read_numbers(const std::string &path) {
    std::vector<double> v;
    if (path.empty()) return v;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    double x;
    while (f >> x) v.push_back(x);
    return v;
}

}  // namespace pgdrv
