"""Writes `bakes.json`: the digest (cases.digest) of the oracle's bake of every case in
cases.CASES, plus how long the oracle took on each.

Run from the repository root after the oracle is built:

    python -m tests.golden.make_golden            # every case
    python -m tests.golden.make_golden small_room # rewrite one case, keep the others
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()

from tests.golden import cases  # noqa: E402

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bakes.json")


def main(names):
    data = {"cases": {}}
    if os.path.exists(PATH):
        with open(PATH) as f:
            data = json.load(f)
    for name in names or list(cases.CASES):
        t0 = time.perf_counter()
        record = cases.digest(cases.oracle_bake(name))
        record["oracle_seconds"] = round(time.perf_counter() - t0, 2)
        data["cases"][name] = record
        print(f"{name}: {len(record['meshes'])} meshes, {record['stats']['rays']} rays, "
              f"{record['oracle_seconds']} s", flush=True)
    data["cases"] = {k: data["cases"][k] for k in cases.CASES if k in data["cases"]}
    data["source"] = "oracle/ (binary32 mode; refined mode at the default epsilon for refined cases)"
    with open(PATH, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:])
