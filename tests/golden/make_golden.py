"""Regenerate the golden fixtures from the reference GRGL itself.

Run after ``oracle/build_ref.sh`` has compiled the reference into oracle/_ref (it also links
the reference checkout there as oracle/_ref/src and its Python package as oracle/_ref/pygrgl):

    python tests/golden/make_golden.py

Produces, next to this script:
  t200.grg / t200.npz         reference constructor on test/endtoend/input/test-200-samples.vcf.gz,
                              and pygrgl.matmul outputs for seeded inputs (all dtypes and options);
                              the UP int32 ones output is checked against the reference's own golden
                              allele counts, test/endtoend/expect/test-200-samples.freq.txt
  t200miss.grg / t200miss.npz the same for test-200-samples.miss.igd (missingness nodes, `miss`)
  wt_n1000_m10000.grg / wt_n1000_m10000.npz         the seeded window-tree genotypes (N=1,000 haplotypes, M=10,000 variants,
                              seed 42) written as VCF and built by the reference constructor, with the
                              reference outputs of DOWN int32 ones, DOWN f64 N(0,1) and UP f64 N(0,1)
Inputs are regenerated in the tests from the seeds stored in each .npz.
"""
from __future__ import annotations

import gzip
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = ROOT / "oracle" / "_ref" / "src"
sys.path[:0] = [str(ROOT / "oracle" / "_ref"), str(ROOT)]

import pygrgl  # noqa: E402  (the reference module built by oracle/build_ref.sh)

from tests.golden.cases import cases_for  # noqa: E402


def construct(src: Path, dst: Path):
    out = subprocess.run([str(ROOT / "oracle" / "_ref" / "ref_construct"), str(src), str(dst)], check=True,
                         capture_output=True, text=True)
    print(out.stdout.strip())


def record(grg_path: Path, npz_path: Path, extra: dict, profile: str):
    g = pygrgl.load_immutable_grg(str(grg_path))
    results = {}
    meta = []
    for name, case in cases_for(g.num_samples, g.num_mutations, g.num_nodes, g.ploidy, has_miss=bool(extra.get("miss")),
                                profile=profile):
        V, direction, kw = case
        kw = dict(kw)
        miss = kw.pop("miss", None)
        if miss is not None:
            miss = miss.copy()
        out = pygrgl.matmul(g, V, pygrgl.TraversalDirection(direction), miss=miss, **kw)
        results[name] = out
        if miss is not None and direction == 2:
            results[name + "__miss"] = miss
        meta.append(name)
    results["__meta__"] = np.frombuffer(json.dumps({"cases": meta, "profile": profile, **extra}).encode(), dtype=np.uint8)
    np.savez_compressed(npz_path, **results)
    print(f"{npz_path.name}: {len(meta)} cases")


def write_vcf(X: np.ndarray, path: Path):
    """Phased diploid VCF of an N x M 0/1 matrix (haplotypes 2i, 2i+1 = individual i)."""
    N, M = X.shape
    with gzip.open(path, "wt") as f:
        f.write("##fileformat=VCFv4.2\n##contig=<ID=1>\n")
        f.write("#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t" +
                "\t".join(f"I{i}" for i in range(N // 2)) + "\n")
        for j in range(M):
            col = X[:, j]
            gts = "\t".join(f"{col[2 * i]}|{col[2 * i + 1]}" for i in range(N // 2))
            f.write(f"1\t{j + 1}\t.\tA\tC\t.\tPASS\t.\tGT\t{gts}\n")


def main():
    if sys.argv[1:] == ["--window-tree-only"]:
        # re-record the window-tree fixture's outputs from its existing .grg
        record(HERE / "wt_n1000_m10000.grg", HERE / "wt_n1000_m10000.npz",
               {"generator": "window_tree N=1000 M=10000 seed=42 window=100"}, "full")
        return
    # 1. the reference's 200-sample test input
    t200 = HERE / "t200.grg"
    construct(REF / "test/endtoend/input/test-200-samples.vcf.gz", t200)
    g = pygrgl.load_immutable_grg(str(t200))
    counts = pygrgl.matmul(g, np.ones((1, g.num_samples), dtype=np.int32), pygrgl.TraversalDirection.UP)[0]
    freq = np.loadtxt(REF / "test/endtoend/expect/test-200-samples.freq.txt", skiprows=1, usecols=3, dtype=np.int64)
    assert np.array_equal(counts, freq), "reference UP ones disagrees with its own freq.txt"
    record(t200, HERE / "t200.npz", {"freq_pinned": True}, "full")

    # 2. missing data
    t200m = HERE / "t200miss.grg"
    construct(REF / "test/endtoend/input/test-200-samples.miss.igd", t200m)
    record(t200m, HERE / "t200miss.npz", {"miss": True}, "miss")

    # 3. seeded window-tree genotypes (N=1,000, M=10,000) -> VCF -> reference constructor
    import oracle
    import grgl_gb300

    direct = grgl_gb300.window_tree_grg(1000, 10000, seed=42)
    a = direct.export_arrays()
    og = oracle.OracleGraph(num_samples=1000, ploidy=2, down_off=a["down_off"], down_adj=a["down_adj"],
                            mut_node=a["mut_node"])
    X = og.dense_X().astype(np.int8)
    assert X.max() <= 1, "window-tree genotypes must be 0/1"
    vcf = Path("/tmp/grgx_wt_n1000_m10000.vcf.gz")
    write_vcf(X, vcf)
    construct(vcf, HERE / "wt_n1000_m10000.grg")
    record(HERE / "wt_n1000_m10000.grg", HERE / "wt_n1000_m10000.npz", {"generator": "window_tree N=1000 M=10000 seed=42 window=100",
                                                  "nnz": int(X.sum())}, "full")


if __name__ == "__main__":
    main()
