"""Summarise an ncu launch list (``--metrics gpu__time_duration.sum --csv``):
launches, total time and share per kernel.  Usage:
    python -m plantfem_gb300.ncu_summary launches.csv [top]
"""
import collections
import csv
import sys

SCALE = {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0, "ms": 1e3, "msecond": 1e3}


def summarise(path, top=20):
    with open(path) as f:
        lines = [ln for ln in f if ln.startswith('"')]
    tot = collections.defaultdict(lambda: [0, 0.0])
    for row in csv.DictReader(lines):
        if row.get("Metric Name") != "gpu__time_duration.sum":
            continue
        us = float(row["Metric Value"].replace(",", "")) * SCALE[row["Metric Unit"]]
        t = tot[row["Kernel Name"]]
        t[0] += 1
        t[1] += us
    T = sum(v[1] for v in tot.values())
    out = [f"{'launches':>8} {'total ms':>10} {'share':>6}  kernel"]
    for k, (n, t) in sorted(tot.items(), key=lambda x: -x[1][1])[:top]:
        out.append(f"{n:8d} {t / 1e3:10.2f} {100 * t / T:5.1f}%  {k.split('(')[0]}")
    out.append(f"{sum(v[0] for v in tot.values()):8d} {T / 1e3:10.2f} 100.0%  (all kernels)")
    return "\n".join(out)


if __name__ == "__main__":
    print(summarise(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 20))
