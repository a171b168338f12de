"""Host-side helpers of bench.py that need no GPU: the sysfs CPU-list parser behind the
host-affinity binding of the host-buffer legs, and the affinity context's restore."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_parse_cpulist():
    assert bench.parse_cpulist("0-3,8,10-11\n") == {0, 1, 2, 3, 8, 10, 11}
    assert bench.parse_cpulist("5") == {5}
    assert bench.parse_cpulist("") == set()


def test_host_affinity_restores_the_callers_cpus():
    before = os.sched_getaffinity(0)
    aff = bench.HostAffinity(0)
    aff.cpus = {min(before)}  # as if the GPU's node held only this CPU
    with aff:
        assert os.sched_getaffinity(0) == {min(before)}
    assert os.sched_getaffinity(0) == before
    assert "1 CPUs local" in aff.note()
    none = bench.HostAffinity(0)
    none.cpus = None
    with none:
        assert os.sched_getaffinity(0) == before
    assert none.note().startswith("not bound")
