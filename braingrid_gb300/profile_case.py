"""Run a benchmark workload for a few steps, for profilers (ncu) to capture its kernels.

    python -m braingrid_gb300.profile_case [--workload c1|c2] [--steps 20] [--flush]
"""
import argparse

from . import workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--flush", action="store_true", help="evict L2 before every step")
    ap.add_argument("--workload", default="c1", choices=["c1", "c2"])
    a = ap.parse_args()
    flush = (256 << 20) if a.flush else 0
    if a.workload == "c1":
        spec, net = workloads.build()
        net.bench_steps(a.steps, flush)
        print("steps", a.steps, "synapses", net.total_synapses(), "error_word", net.error_word)
        assert net.error_word == 0
    else:
        from . import lib as bg
        nets = [workloads.build_member(w)[1] for w in workloads.c2_members()]
        batch = bg.Batch(nets)
        batch.bench_steps(a.steps, flush)
        S = sum(n.total_synapses() for n in nets)
        print("steps", a.steps, "networks", len(nets), "synapses", S)
        assert max(n.error_word for n in nets) == 0


if __name__ == "__main__":
    main()
