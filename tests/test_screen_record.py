"""The packed 16-byte screen record (pack_screen / unpack_screen / screen_with_ev in
acvd_gb300/csrc/state.cuh): its fields round-trip, the evaluation sweep can be replaced
without touching the rest, and -1 ("no evaluation without a proposal") and the largest
ids and sweeps a record holds survive.  The helpers are host-and-device functions, so
this compiles them with nvcc into a host program and runs it on the CPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "acvd_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include "state.cuh"
using namespace acvd;

static int fails = 0;
static void check(bool ok, const char* what, long long a) {
    if (!ok) { std::printf("FAIL %s %lld\n", what, a); fails++; }
}

int main() {
    unsigned long long x = 88172645463325252ull;
    auto rnd = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return x; };
    const int ids[] = {0, 1, 12345, kCacheClusters - 1};
    const int evs[] = {-1, 0, 1, 255, 256, 65535, 65536, (1 << 24) - 1, 1 << 24, kCacheSweeps - 1};
    for (int trial = 0; trial < 20000; trial++) {
        const int L = trial < 4 ? ids[trial] : (int)(rnd() % kCacheClusters);
        const int t0 = (int)(rnd() % kCacheClusters), t1 = (int)(rnd() % kCacheClusters);
        const int t2 = trial < 4 ? ids[3 - trial] : (int)(rnd() % kCacheClusters);
        const int meta = (int)(rnd() % 16);
        const int ev = trial < 10 ? evs[trial] : (int)(rnd() % (unsigned)kCacheSweeps) - 1;
        const int4 c = pack_screen(L, t0, t1, t2, meta, ev);
        const Screen s = unpack_screen(c);
        check(s.L == L, "L", L);
        check(s.t[0] == t0 && s.t[1] == t1 && s.t[2] == t2, "targets", trial);
        check(s.n == (meta & 3) && s.conn_known == ((meta & 4) != 0) && s.conn_ok == ((meta & 8) != 0), "meta", meta);
        check(s.ev == ev, "ev", ev);
        const int ev2 = (int)(rnd() % (unsigned)kCacheSweeps) - 1;
        const Screen s2 = unpack_screen(screen_with_ev(c, ev2));
        check(s2.ev == ev2, "ev2", ev2);
        check(s2.L == L && s2.t[0] == t0 && s2.t[1] == t1 && s2.t[2] == t2 && s2.n == s.n &&
                  s2.conn_known == s.conn_known && s2.conn_ok == s.conn_ok,
              "fields kept", trial);
    }
    std::printf("%s\n", fails ? "FAILED" : "OK");
    return fails ? 1 : 0;
}
"""


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_screen_record_round_trip(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "screen_record.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "screen_record"
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
