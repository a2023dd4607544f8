"""Run a benchmark workload for a few steps, for profilers (ncu) to capture its kernels.

    python -m braingrid_gb300.profile_case [--steps 20] [--flush]
"""
import argparse

from . import workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--flush", action="store_true", help="evict L2 before every step")
    a = ap.parse_args()
    spec, net = workloads.build()
    net.bench_steps(a.steps, (256 << 20) if a.flush else 0)
    print("steps", a.steps, "synapses", net.total_synapses(), "error_word", net.error_word)
    assert net.error_word == 0


if __name__ == "__main__":
    main()
