// Autotuner cache of the TI batches: one JSON object per line,
//   {"key": "<batch key>", "form": F, "simt_threads": T, "tc_steps": S, "ms_per_step": M}
// The last record of a key wins; lines that do not parse are skipped.  Plain
// C++ (no CUDA), so that the host tests can compile it on its own.
#pragma once
#include <cstdio>
#include <cstring>
#include <string>

#include "pimdgpu.h"

namespace pg {

struct TuneChoice {
    int form = PG_FORM_AUTO, simt_threads = 0, tc_steps = 0;
    double ms_per_step = 0.0;
};

inline bool tune_int(const char *line, const char *name, int &v) {
    const char *q = strstr(line, name);
    return q && sscanf(q + strlen(name), " : %d", &v) == 1;
}

inline bool tune_lookup(const std::string &path, const std::string &key, TuneChoice &c) {
    FILE *fp = fopen(path.c_str(), "r");
    if (!fp) return false;
    const std::string kq = "\"key\": \"" + key + "\"";
    char line[2048];
    bool found = false;
    while (fgets(line, sizeof(line), fp))  // the last record of a key wins
        if (strstr(line, kq.c_str())) {
            TuneChoice t;
            if (tune_int(line, "\"form\"", t.form) && tune_int(line, "\"simt_threads\"", t.simt_threads) &&
                tune_int(line, "\"tc_steps\"", t.tc_steps)) {
                c = t;
                found = true;
            }
        }
    fclose(fp);
    return found;
}

inline void tune_record(const std::string &path, const std::string &key, const TuneChoice &c) {
    FILE *fp = fopen(path.c_str(), "a");
    if (!fp) return;  // a cache that cannot be written is not an error
    fprintf(fp, "{\"key\": \"%s\", \"form\": %d, \"simt_threads\": %d, \"tc_steps\": %d, \"ms_per_step\": %.6g}\n",
            key.c_str(), c.form, c.simt_threads, c.tc_steps, c.ms_per_step);
    fclose(fp);
}

}  // namespace pg
