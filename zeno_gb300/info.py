"""Capacity report for the GPU: `zeno info` (src/main.rs:1001-1082) with HBM
in place of RAM: the budget of `zc_device_budget` is 0.75 x the device memory
(the total HBM, or ZENO_MEM_BYTES pretending to be a smaller device). The
JSON keeps zeno's schema v1 keys (`ram_bytes` = that device memory, `cores` =
SMs) and adds the GPU's own.

  python -m zeno_gb300.info [--json]
"""

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from zeno_gb300 import backend as zb  # noqa: E402

FRACTION = 0.75


def human(b: int) -> str:
    """Binary units like the reference's human_bytes."""
    v, u = float(b), 0
    units = ["B", "KiB", "MiB", "GiB", "TiB"]
    while v >= 1024 and u < len(units) - 1:
        v /= 1024
        u += 1
    return ("%.0f %s" if u == 0 else "%.1f %s") % (v, units[u])


def capacity(budget: int, precision: int) -> dict:
    n = zb.max_qubits(budget, precision)
    return {"max_qubits": n, "state_bytes": zb.state_bytes(n, precision),
            "next_qubit_bytes": zb.state_bytes(n + 1, precision)}


def report() -> dict:
    d = zb.device_info()
    budget = zb.device_budget(FRACTION)
    return {"schema_version": 1, "chip": d["name"], "cores": d["sms"], "ram_bytes": zb.device_memory(),
            "sms": d["sms"],
            "compute_capability": d["compute_capability"], "hbm_bytes": d["hbm_bytes"],
            "available_now_bytes": d["free_bytes"], "l2_bytes": d["l2_bytes"], "budget_bytes": budget,
            "budget_fraction": FRACTION,
            "precisions": {"f64": capacity(budget, 64), "f32": capacity(budget, 32)},
            "overrides": ["ZENO_MEM_BYTES"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--json", action="store_true")
    a = ap.parse_args()
    r = report()
    if a.json:
        print(json.dumps(r, indent=2))
        return
    print("zeno_gb300 · %s (sm_%s, %d SMs)" % (r["chip"], r["compute_capability"].replace(".", ""), r["sms"]))
    print("  memory  %s HBM · free now ~%s · budget %s (%.0f%% of HBM)" % (
        human(r["hbm_bytes"]), human(r["available_now_bytes"]), human(r["budget_bytes"]), FRACTION * 100))
    print()
    print("  %-10s %10s %12s %18s" % ("precision", "max qubits", "state size", "next qubit needs"))
    for p in ("f64", "f32"):
        c = r["precisions"][p]
        print("  %-10s %10d %12s %18s" % (p, c["max_qubits"], human(c["state_bytes"]), human(c["next_qubit_bytes"])))
    print()
    print("ZENO_MEM_BYTES overrides the device memory the budget is taken from")


if __name__ == "__main__":
    main()
