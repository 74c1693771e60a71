"""The autotuner's JSON-lines cache (pimd-tunneling_gb300/csrc/pg_tune.h), compiled
on its own with the host C++ compiler: records round-trip, the last record of a
key wins, other keys and malformed lines are skipped, a missing file is a miss."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r'''
#include <cstdio>
#include <cstdlib>
#include "pg_tune.h"
int main(int argc, char **argv) {
    const std::string path = argv[1], op = argv[2], key = argv[3];
    pg::TuneChoice c;
    if (op == "put") {
        c.form = atoi(argv[4]);
        c.simt_threads = atoi(argv[5]);
        c.tc_steps = atoi(argv[6]);
        c.ms_per_step = 0.5;
        pg::tune_record(path, key, c);
        return 0;
    }
    if (!pg::tune_lookup(path, key, c)) {
        std::printf("miss\n");
        return 0;
    }
    std::printf("%d %d %d\n", c.form, c.simt_threads, c.tc_steps);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("tune")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "csrc"), "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    return str(exe)


def _run(exe, *args):
    return subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True,
                          check=True).stdout.strip()


def test_cache_round_trip_and_last_record_wins(harness, tmp_path):
    f = tmp_path / "tune.jsonl"
    assert _run(harness, f, "get", "A") == "miss"  # no file
    _run(harness, f, "put", "A", 3, 0, 0)
    _run(harness, f, "put", "B", 2, 64, 0)
    assert _run(harness, f, "get", "A") == "3 0 0"
    assert _run(harness, f, "get", "B") == "2 64 0"
    _run(harness, f, "put", "A", 2, 128, 0)  # a later record of the same key
    assert _run(harness, f, "get", "A") == "2 128 0"
    assert _run(harness, f, "get", "C") == "miss"
    assert len(f.read_text().splitlines()) == 3


def test_cache_skips_malformed_lines_and_prefix_keys(harness, tmp_path):
    f = tmp_path / "tune.jsonl"
    f.write_text('not json\n{"key": "A", "form": "x"}\n{"key": "AB", "form": 3, "simt_threads": 0, '
                 '"tc_steps": 0}\n')
    assert _run(harness, f, "get", "A") == "miss"  # the malformed record of A, and the key AB, do not count
    _run(harness, f, "put", "A", 2, 32, 0)
    assert _run(harness, f, "get", "A") == "2 32 0"
    assert _run(harness, f, "get", "AB") == "3 0 0"
