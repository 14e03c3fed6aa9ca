"""Summary of a kernel timeline written by the diagnostic build.

A build with MECH_TRACE=1 in the environment (``picgo_gb300.build``) makes
every kernel block append one record (start ns, end ns, kernel id << 32 | block)
to a device buffer, and ``mech_minimize`` writes the records to the file named
by MECH_TRACE_FILE.  The single-block finalizers also record sections of their
own work (partial loads, block reduction, the CG step logic in thread 0).

    python -m picgo_gb300.timeline FILE [ITERATIONS [WINDOW]]

prints the wall and busy time of the timeline, the time at each concurrency
level, and per kernel: launches (blocks of one kernel whose records overlap or
follow within `gap` ns form one launch), total, share, mean, median and max
duration, and per CG iteration when ITERATIONS is given; WINDOW > 0 also lists
that many launches from the middle of the timeline.
"""
from __future__ import annotations

import collections
import sys

import numpy as np

# kernel ids, in the order of mech_internal.cuh's TraceKernel
NAMES = {
    1: "fil_energy", 2: "fil_force", 3: "gather", 4: "fin_force", 5: "fin_energy", 6: "fil_energy_bulk",
    7: "fil_force_bulk", 8: "direction_mx", 9: "bond", 10: "direction", 11: "fin_direction", 12: "reset",
    13: "recover_maxabs", 14: "recover_move", 15: "backup", 16: "exvol_fb_force", 17: "exvol", 18: "exvol_ext",
    19: "exvol_tail", 20: "body_head", 21: "gather_mx",
    22: "fin_energy: loads", 23: "fin_energy: reduce", 24: "fin_energy: step", 25: "fin_force: loads",
    26: "fin_force: reduce", 27: "fin_force: step", 28: "tail_coop",
}
SECTIONS = set(range(22, 28))


def load(path: str):
    a = np.fromfile(path, dtype=np.uint64).reshape(-1, 3)
    return (a[:, 0].astype(np.int64), a[:, 1].astype(np.int64), (a[:, 2] >> 32).astype(np.int64),
            (a[:, 2] & 0xFFFFFFFF).astype(np.int64))


def launches(t0, t1, kid, gap: int = 300):
    """(kernel, start, end, blocks) per launch, in start order."""
    out = []
    for k in np.unique(kid):
        m = kid == k
        o = np.argsort(t0[m], kind="stable")
        a0, a1 = t0[m][o], t1[m][o]
        s, hi = 0, a1[0]
        for i in range(1, len(a0) + 1):
            if i == len(a0) or a0[i] > hi + gap:
                out.append((int(k), int(a0[s:i].min()), int(a1[s:i].max()), int(i - s)))
                if i < len(a0):
                    s, hi = i, a1[i]
            else:
                hi = max(hi, a1[i])
    out.sort(key=lambda x: x[1])
    return out


def summarize(path: str, iterations: float | None = None, window: int = 0) -> str:
    t0, t1, kid, _ = load(path)
    L = launches(t0, t1, kid)
    kernels = [x for x in L if x[0] not in SECTIONS]
    T0, T1 = min(x[1] for x in kernels), max(x[2] for x in kernels)
    wall = (T1 - T0) / 1e3
    events = sorted([(x[1], 1) for x in kernels] + [(x[2], -1) for x in kernels])
    busy, depth, last, conc = 0, 0, None, collections.Counter()
    for t, d in events:
        if last is not None and depth > 0:
            busy += t - last
            conc[min(depth, 4)] += t - last
        depth += d
        last = t
    lines = [f"records {len(t0)}  launches {len(kernels)}  wall {wall:.1f} us  busy {busy / 1e3:.1f} us  "
             f"idle {wall - busy / 1e3:.1f} us",
             "concurrency (us): " + str({k: round(v / 1e3, 1) for k, v in sorted(conc.items())})]
    per = collections.defaultdict(list)
    for k, a, b, _ in L:
        per[k].append((b - a) / 1e3)
    tot = sum(sum(v) for k, v in per.items() if k not in SECTIONS)
    head = f"{'kernel':20s} {'launch':>7s} {'sum us':>9s} {'share':>6s} {'mean':>7s} {'med':>7s} {'max':>7s}"
    lines.append(head + ("  per-iter" if iterations else ""))
    for k, v in sorted(per.items(), key=lambda kv: (kv[0] in SECTIONS, -sum(kv[1]))):
        v = np.array(v)
        share = "" if k in SECTIONS else f"{v.sum() / tot:6.1%}"
        extra = f"  {v.sum() / iterations:8.1f}" if iterations else ""
        lines.append(f"{NAMES.get(k, str(k)):20s} {len(v):7d} {v.sum():9.1f} {share:>6s} {v.mean():7.2f} "
                     f"{np.median(v):7.2f} {v.max():7.2f}" + extra)
    if iterations:
        lines.append(f"wall per iteration {wall / iterations:.1f} us; busy per iteration {busy / 1e3 / iterations:.1f} us")
    if window > 0:
        off = len(kernels) // 2
        base = kernels[off][1]
        for k, a, b, nb in kernels[off:off + window]:
            lines.append(f"{(a - base) / 1e3:9.2f} {(b - base) / 1e3:9.2f} {(b - a) / 1e3:7.2f} "
                         f"{NAMES.get(k, str(k)):16s} blocks={nb}")
    return "\n".join(lines)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    print(summarize(sys.argv[1], float(sys.argv[2]) if len(sys.argv) > 2 else None,
                    int(sys.argv[3]) if len(sys.argv) > 3 else 0))
