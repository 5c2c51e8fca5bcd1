"""The engine's arena sizing policy (libfluid_gb300/csrc/arena_policy.h),
checked on the host: a small C++ driver compiled against the header answers
plan_arena queries.

* Whatever it grants fits the byte budget and covers what was asked.
* It refuses exactly the requests that cannot fit (over budget), and a large
  arena that could only grow by less than an eighth (at budget: the caller
  waits for scenes to leave).
* Without a budget growth is geometric (x1.5).
* A server-like sequence of admissions and departures under a budget grows
  the arena a handful of times, not once per admission.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OK, OVER, AT_BUDGET = 0, 1, 2
BPP = 288

DRIVER = r"""
#include "arena_policy.h"
#include <cstdio>
int main() {
    unsigned long long a, b, c, d, e, f;
    while (std::scanf("%llu %llu %llu %llu %llu %llu", &a, &b, &c, &d, &e, &f) == 6) {
        const sph::ArenaPlan p = sph::plan_arena(a, b, c, d, e, f);
        std::printf("%llu %llu %d\n", (unsigned long long)p.parts, (unsigned long long)p.cells, p.status);
        std::fflush(stdout);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("arena")
    (d / "driver.cpp").write_text(DRIVER)
    exe = d / "driver"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I",
                    os.path.join(ROOT, "libfluid_gb300", "csrc"), str(d / "driver.cpp"), "-o", str(exe)], check=True)

    proc = subprocess.Popen([str(exe)], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True, bufsize=1)

    def run(queries):
        out = []
        for q in queries:
            proc.stdin.write(" ".join(str(int(v)) for v in q) + "\n")
            proc.stdin.flush()
            out.append(tuple(int(x) for x in proc.stdout.readline().split()))
        return out
    yield run
    proc.stdin.close()
    proc.wait(timeout=10)


def test_random_queries(plan):
    rng = np.random.default_rng(5)
    queries = []
    for _ in range(20000):
        pcap = int(rng.choice([0, int(rng.integers(1, 1 << 12)), int(rng.integers(1 << 20, 1 << 27))]))
        ccap = int(rng.integers(0, 1 << 26))
        parts = int(max(0, pcap + rng.integers(-(1 << 20), 1 << 22)))
        cells = int(max(0, ccap + rng.integers(-(1 << 20), 1 << 22)))
        limit = int(rng.choice([0, int(rng.integers(1 << 30, 1 << 36))]))
        queries.append((parts, cells, pcap, ccap, limit, BPP))
    for (parts, cells, pcap, ccap, limit, bpp), (np_, nc, st) in zip(queries, plan(queries)):
        need = max(parts, pcap) * bpp + max(cells, ccap) * 8
        if limit and need > limit:
            assert st == OVER and (np_, nc) == (pcap, ccap)
            continue
        if st == AT_BUDGET:
            assert limit and pcap >= (1 << 20) and parts > pcap and (np_, nc) == (pcap, ccap)
            # growing by an eighth would not have left room for the cells
            assert (pcap + pcap // 8) * bpp + max(cells, ccap) * 8 + limit // 32 > limit
            continue
        assert st == OK
        assert np_ >= max(parts, pcap) and nc >= max(cells, ccap)
        if limit:
            assert np_ * bpp + nc * 8 <= limit
        else:
            assert np_ == (max(parts, pcap + pcap // 2) if parts > pcap else pcap)
            assert nc == (max(cells, ccap + ccap // 2) if cells > ccap else ccap)
        if parts > pcap >= (1 << 20):
            assert np_ >= pcap + pcap // 8


def test_admission_sequence_grows_rarely(plan):
    """Scenes of 1k-262k particles arrive and leave under a 64 GB budget;
    the arena's high-water mark is what an admission asks for."""
    rng = np.random.default_rng(6)
    limit = 64 << 30
    cells_per_particle = 2
    pcap = ccap = 0
    live, grows, waits, admitted = [], 0, 0, 0
    for _ in range(10000):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(262144))))
        # departures: a scene leaves with probability 1/2 per admission
        if live and rng.random() < 0.5:
            live.pop(int(rng.integers(len(live))))
        parts = sum(live) + n
        cells = parts * cells_per_particle
        (np_, nc, st), = plan([(parts, cells, pcap, ccap, limit, BPP)])
        if st != OK:
            waits += 1
            if live:
                live.pop(0)
            continue
        if np_ > pcap:
            grows += 1
        pcap, ccap = np_, nc
        assert pcap * BPP + ccap * 8 <= limit
        live.append(n)
        admitted += 1
    assert admitted > 9000
    assert grows <= 40, grows
