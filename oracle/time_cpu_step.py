"""Times the CPU time step of the C2 workload (the layer over a half-space, free
surface on top, 30-point supergrid elsewhere, moment source) on the reference's own
kernels (oracle/_ref, compiled from the reference sources where they are present)
and on the oracle's restatement of them, with the same OpenMP thread count.  The
ratio tells how far the port that bench.py's reference arm times on machines
without the reference tree is from the reference itself.

    python oracle/time_cpu_step.py [n] [steps]      (defaults 256 and 4)

TEST INFRASTRUCTURE ONLY: nothing in the product imports it.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 256
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 4
    import bench
    from oracle import oracle as O
    if not O.ref_available():
        if O.reference_src() is None:
            sys.exit("the reference's kernels are not built here (no reference tree)")
        O.build(ref=True)
    out = {}
    for which in ("ref", "oracle"):
        rate, el, kind, cores = bench.cpu_rate(n, steps, 1, which=which)
        out[which] = rate
        print(f"{kind:9s} {n}^3, {steps} steps, {cores} threads: {rate / 1e6:8.2f} M grid-pt-steps/s "
              f"({el / steps:.3f} s per step)")
    print(f"port / reference = {out['oracle'] / out['ref']:.3f}")


if __name__ == "__main__":
    main()
