"""Extract the reference's stored known answers into reference_golden.json.

Reads (from a checkout of RealSpace_ExactDiagonalization, given as the first
argument or in the environment variable SED_REFERENCE_ROOT):
  * benchmark/benchmark_data/benchmark_raw.csv -- per (model, size, mode):
    n_site, n_filled, full_dim, n_orbits, |G|, sector_dim and the ground
    energy of the k=(0,0) sector;
  * doc/design.ipynb cell outputs -- the colex rank table for N=4, k=2, the
    LinTable / rank agreement over C(12,3), and the Haldane 2x3 counts
    (orbits, full basis, sector dim, nnz(H), projection-table entries).
The JSON is committed; tests read only the JSON.  Re-run with
``python tests/golden/make_golden.py <reference_root>``.
"""
import csv
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SED_REFERENCE_ROOT", "")
if not ROOT:
    sys.exit("usage: make_golden.py <reference_root> (or set SED_REFERENCE_ROOT)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")


def bench_rows():
    path = os.path.join(ROOT, "benchmark", "benchmark_data", "benchmark_raw.csv")
    rows = []
    with open(path) as f:
        for r in csv.DictReader(f):
            rows.append({
                "model": r["model"], "label": r["label"], "n_site": int(r["n_site"]), "n_filled": int(r["n_filled"]),
                "full_dim": int(r["full_dim"]), "n_orbits": int(r["n_orbits"]), "n_group": int(r["n_group"]),
                "sector_dim": int(r["sector_dim"]), "mode": r["mode"], "elapsed_s": float(r["elapsed_s"]),
                "energy": float(r["energy"]), "source": "benchmark/benchmark_data/benchmark_raw.csv",
            })
    return rows


def notebook_outputs():
    nb = json.load(open(os.path.join(ROOT, "doc", "design.ipynb")))
    texts = {}
    for i, c in enumerate(nb["cells"]):
        out = []
        for o in c.get("outputs", []):
            t = o.get("text") or o.get("data", {}).get("text/plain")
            if t:
                out.append("".join(t))
        if out:
            texts[i] = "\n".join(out)
    return texts


def main():
    texts = notebook_outputs()
    g = {"benchmark_raw": bench_rows()}
    # colex rank table (cell 22)
    t22 = texts[22]
    g["colex_rank_n4_k2"] = [[int(a), int(b)] for a, b in re.findall(r"^\s*(\d+) = [01]+\s+->\s+rank = (\d+)", t22,
                                                                        re.M)]
    g["rank_0b1010"] = int(re.search(r"rank\(0b1010\) = (\d+)", t22).group(1))
    # LinTable (cell 24)
    t24 = texts[24]
    g["lin_table_12_3"] = {
        "left_len": int(re.search(r"lengths: (\d+)/(\d+)", t24).group(1)),
        "right_len": int(re.search(r"lengths: (\d+)/(\d+)", t24).group(2)),
        "n_right": int(re.search(r"n_right = (\d+)", t24).group(1)),
        "lin_index_0b1010_n4k2": int(re.search(r"lin_index\(0b1010\) = (\d+)", t24).group(1)),
        "mismatches_over_220": int(re.search(r"mismatches over 220 masks: (\d+)", t24).group(1)),
    }
    # Haldane 2x3 catalog / sector / H counts (cells 26 and 43)
    t26, t43 = texts[26], texts[43]
    g["haldane_2x3"] = {
        "n_orbits": int(re.search(r"n_orbits = (\d+)", t26).group(1)),
        "full_basis": int(re.search(r"full basis C\(12,3\) = (\d+)", t26).group(1)),
        "rep_rank_unset": int(re.search(r"unset = (\d+)", t26).group(1)),
        "sector_dim": int(re.search(r"sector dim = (\d+)", t43).group(1)),
        "nnz_H": int(re.search(r"nnz\(H\) = (\d+)", t43).group(1)),
        "projection_entries": int(re.search(r"projection table entries = (\d+)", t43).group(1)),
        "source": "doc/design.ipynb cells 26, 43",
    }
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT, len(g["benchmark_raw"]), "benchmark rows")


if __name__ == "__main__":
    main()
