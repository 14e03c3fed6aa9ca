"""A bounded piece of the minimization, for profilers and quick timings.

    python -m picgo_gb300.cg_probe --workload c2 --precision mixed --energy-calls 40
    python -m picgo_gb300.cg_probe --workload c2 --precision mixed --evals 2
    python -m picgo_gb300.cg_probe --workload c2 --precision mixed --forces 3

The first form runs neighbor-list rebuild + Polak-Ribiere CG from the seeded
start until `--energy-calls` energy calls (a launch-list target: every kernel
of real CG iterations); the second launches each evaluation kernel `--evals`
times through mech_profile; the third makes only `--forces` mech_forces calls
(or `--energies` mech_energy calls), so that a profiler's first matching
launches are those of one evaluation kind.  Each prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

from . import Engine, cg_params, make_network


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c2", help="network config name (c1, c2, c5)")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--energy-calls", type=int, default=40)
    ap.add_argument("--evals", type=int, default=0, help="profile mode: launches per evaluation kernel")
    ap.add_argument("--forces", type=int, default=0, help="only this many mech_forces calls")
    ap.add_argument("--energies", type=int, default=0, help="only this many mech_energy calls")
    ap.add_argument("--autotune", action="store_true", help="run the autotuner first")
    args = ap.parse_args(argv)
    net = make_network(args.workload, seed=args.seed)
    out = {"workload": args.workload, "precision": args.precision, "n_beads": net.n_beads}
    with Engine(args.precision) as eng:
        eng.set_network(net)
        if args.autotune:
            out["tuning"] = eng.autotune()
        out["lists"] = eng.rebuild()
        if args.forces > 0 or args.energies > 0:
            for _ in range(args.forces):
                f = eng.forces()
            for _ in range(args.energies):
                e = eng.energies()[1]
            out["calls"] = {"forces": args.forces, "energies": args.energies}
        elif args.evals > 0:
            out["profile"] = eng.profile(args.evals)
        else:
            t0 = time.perf_counter()
            r = eng.minimize(cg_params(energy_rel_tol=0.0, energy_call_limit=args.energy_calls,
                                       force_call_limit=1_000_000))[0]
            out["seconds"] = round(time.perf_counter() - t0, 4)
            out.update({k: r[k] for k in ("num_iter", "num_force_call", "num_energy_eval", "grad_inf_norm",
                                          "status")})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
