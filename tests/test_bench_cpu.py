"""bench.py host pieces: the roofline traffic it reads from the committed ncu
summaries, and the workload definitions."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_profile_traffic_lines():
    import bench
    assert bench.profile_traffic('k_lu32') == (35300.0, os.path.join('profiles', 'k_lu32_64cols.md'))
    assert bench.profile_traffic('k_rates')[0] == 17600.0
    assert bench.profile_traffic('no_such_kernel') == (None, None)


def test_workloads():
    import argparse
    import bench
    a = argparse.Namespace(workload='c2', ncols=None, converge=False)
    net, specs = bench._workload(a, 8)
    assert net.ni == 69 and len(specs) == 8
