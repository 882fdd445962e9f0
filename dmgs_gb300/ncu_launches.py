"""Summarise an ncu launch list (``--metrics gpu__time_duration.sum --csv``).

    python -m dmgs_gb300.ncu_launches launches.csv [--marker REGEX --last N]

Prints, per kernel, the launches, the total device time and its share.  With
``--marker``/``--last`` only the launches from the N-th last launch of the
kernel matching REGEX onward are counted (e.g. the timed steps of a bench
run, each of which begins with the same kernel).  ncu serialises launches and
runs them with cold caches, so the shares are the figures to compare with
CUDA-event timings, not the absolute times.
"""
from __future__ import annotations

import argparse
import collections
import csv
import re


def read(path):
    lines = open(path).read().splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.startswith('"ID"'))
    rows = list(csv.reader(lines[start:]))
    hdr, rows = rows[0], rows[1:]
    ki, mi, vi, ui = (hdr.index(k) for k in ("Kernel Name", "Metric Name", "Metric Value", "Metric Unit"))
    out = []
    for r in rows:
        if r[mi] != "gpu__time_duration.sum":
            continue
        scale = {"ns": 1e-6, "us": 1e-3, "usecond": 1e-3, "nsecond": 1e-6, "ms": 1.0, "msecond": 1.0}[r[ui]]
        out.append((short_name(r[ki]), float(r[vi].replace(",", "")) * scale))
    return out


def short_name(full):
    name = full.split("(")[0]
    name = re.sub(r"^void ", "", name)
    name = re.sub(r"dmgs::<unnamed>::", "", name)
    return name.strip()


def summarise(launches, marker=None, last=None):
    if marker is not None:
        idx = [i for i, (n, _) in enumerate(launches) if re.search(marker, n)]
        if last is not None and len(idx) >= last:
            launches = launches[idx[-last]:]
    count = collections.Counter()
    total = collections.defaultdict(float)
    for n, ms in launches:
        count[n] += 1
        total[n] += ms
    grand = sum(total.values()) or 1.0
    return [(n, count[n], total[n], total[n] / grand) for n in sorted(total, key=lambda k: -total[k])]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("csv")
    ap.add_argument("--marker", default=None)
    ap.add_argument("--last", type=int, default=None)
    a = ap.parse_args()
    rows = summarise(read(a.csv), a.marker, a.last)
    print("| kernel | launches | total ms | share |")
    print("|---|---:|---:|---:|")
    for n, c, t, s in rows:
        print(f"| `{n}` | {c} | {t:.3f} | {100 * s:.1f}% |")
    print(f"| **all** | {sum(r[1] for r in rows)} | {sum(r[2] for r in rows):.3f} | 100% |")


if __name__ == "__main__":
    main()
