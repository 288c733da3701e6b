"""The bench_sort and bench_sort_phases drivers (the reference's bench mains,
bench_sort.cpp and bench_sort_phases.cpp, on the GPU): argument handling on
the CPU, and on the GPU every item kind through both buffer placements, the
multi-thread argument form, and every phase table of bench_sort_phases, each
line checked by the driver itself (it exits non-zero on an unsorted result)."""
import json
import os
import subprocess

import pytest

import __graft_entry__ as entry

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "origami-sort_gb300", "bin")


@pytest.fixture(scope="module", autouse=True)
def built():
    entry.build_library()


def run(*args, timeout=300):
    return subprocess.run([os.path.join(BIN, args[0]), *map(str, args[1:])], capture_output=True, text=True,
                          timeout=timeout)


def json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_drivers_built():
    for exe in ("bench_sort", "bench_sort_phases"):
        assert os.access(os.path.join(BIN, exe), os.X_OK)


def test_bench_sort_usage():
    r = run("bench_sort")
    assert r.returncode == 2 and "usage: bench_sort" in r.stderr
    r = run("bench_sort", 20, 4, 2)  # n_threads > 1 needs n_cores and min_k
    assert r.returncode == 2 and "n_cores" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["u32", "u64", "i64", "kv64", "kvu64"])
@pytest.mark.parametrize("device", [False, True])
def test_bench_sort(kind, device):
    args = ["bench_sort", 22, 1, 2, "--kind", kind, "--repeat", 2, "--dist", 3]
    if device:
        args.append("--device")
    r = run(*args)
    assert r.returncode == 0, r.stdout + r.stderr
    (line,) = json_lines(r.stdout)
    assert line["correct"] is True and line["kind"] == kind
    assert line["buffers"] == ("device" if device else "host") and line["mkeys_per_s"] > 0


@pytest.mark.gpu
def test_bench_sort_multi_thread_form():
    r = run("bench_sort", 22, 8, 8, 16, "--repeat", 1, "--dist", 5)
    assert r.returncode == 0, r.stdout + r.stderr
    (line,) = json_lines(r.stdout)
    assert line["correct"] is True and line["min_k"] == 16 and line["n_threads"] == 8


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["u32", "kv64"])
def test_bench_sort_phases(kind):
    r = run("bench_sort_phases", "all", "--kind", kind, "--pow", 22, "--repeat", 1, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = json_lines(r.stdout)
    phases = {l["phase"] for l in lines}
    assert phases == {"phase1", "phase2", "phase3", "phase4"}
    for l in lines:
        assert l["passes"] >= 1 and l["ms"] > 0
    assert sorted(l["min_k"] for l in lines if l["phase"] == "phase4") == [2, 4, 8, 16]
