"""Summarise an ncu launch list (one gpu__time_duration.sum row per kernel launch) per kernel.

    python -m drd_application_gb300.ncu_summary launches.csv [top]

Prints, per kernel name: launches, total time, mean time and share of the total (ncu times
are cold-cache and serialised, so the shares are what to compare with live timings).
"""
import collections
import csv
import sys


def summarize(path, top=25):
    rows = []
    with open(path, newline="") as f:
        lines = [ln for ln in f if ln.startswith('"')]
    rd = csv.DictReader(lines)
    for r in rd:
        if r.get("Metric Name") != "gpu__time_duration.sum":
            continue
        val = float(r["Metric Value"].replace(",", ""))
        unit = r.get("Metric Unit", "ns")
        scale = {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0, "ms": 1e3, "msecond": 1e3}.get(unit, 1e-3)
        name = r["Kernel Name"].split("(")[0]
        rows.append((name, val * scale))
    agg = collections.defaultdict(lambda: [0, 0.0])
    for name, us in rows:
        agg[name][0] += 1
        agg[name][1] += us
    total = sum(v[1] for v in agg.values())
    out = [f"launches profiled: {len(rows)}   total device time: {total / 1e3:.3f} ms",
           f"{'kernel':70s} {'launches':>9s} {'total_us':>11s} {'mean_us':>9s} {'share':>7s}"]
    for name, (n, us) in sorted(agg.items(), key=lambda kv: -kv[1][1])[:top]:
        out.append(f"{name[:70]:70s} {n:9d} {us:11.1f} {us / n:9.2f} {100 * us / total:6.1f}%")
    return "\n".join(out)


if __name__ == "__main__":
    print(summarize(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 25))
