"""Generate tests/golden/belt_ensemble.json: the oracle's time-averaged
statistics of every member of the belt-bed ensemble (tests/belt_ensemble.py),
each member run for 1e5 steps by the FP64 oracle on one core.

    python tests/golden/make_belt_ensemble.py --members 640 --procs 7

Members run in a spawn pool; the output lists per-member averages in member
order, so any prefix of the ensemble can be reused."""
import argparse
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def run_member(j):
    import belt_ensemble as be
    import parity_util as pu
    from oracle import oracle as om
    om.set_threads(1)
    st = be.member_state(j)
    o = pu.oracle_sim(om, st, be.DT, be.LO, be.HI, 1, 0, cell=be.CELL)
    o.set_options(record_pairs=False, keep_contact_map=False)
    v, n, floor = be.walls()
    o.add_triangles(v[~floor], n[~floor])
    o.add_triangles(v[floor], n[floor], motion=be.BELT)
    out, done = [], 0
    for s in be.sample_steps():
        o.steps(s - done)
        done = s
        q = o.state()
        out.append(be.sample(q["x"], q["v"], q["w"], q["r"], q["m"], be.LO[1]))
    return j, np.mean(out, axis=0).tolist(), len(q["r"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=640)
    ap.add_argument("--procs", type=int, default=max(1, (os.cpu_count() or 2) - 1))
    ap.add_argument("--out", default=os.path.join(HERE, "belt_ensemble.json"))
    a = ap.parse_args()
    from oracle import oracle as om
    om.build()
    t0 = time.time()
    res = [None] * a.members
    with mp.get_context("spawn").Pool(a.procs) as pool:
        for j, avg, n in pool.imap_unordered(run_member, range(a.members)):
            res[j] = avg
            assert n == 500, n
            print(f"member {j}: {avg} ({time.time() - t0:.0f} s)", flush=True)
    arr = np.array(res)
    doc = {"generator": "tests/golden/make_belt_ensemble.py", "oracle": "FP64 oracle, one core per member",
           "members": a.members, "stats": ["kinetic_energy", "coordination", "packing"],
           "mean": arr.mean(0).tolist(), "std": arr.std(0, ddof=1).tolist(), "per_member": res}
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=0)
    print("mean", arr.mean(0), "std", arr.std(0, ddof=1), "rel sem", arr.std(0, ddof=1) / np.sqrt(len(arr)) / arr.mean(0))


if __name__ == "__main__":
    main()
