"""Generates the golden vectors under tests/golden/ from the reference itself.

Run in a container that holds the reference sources, naming their checkout
with --ref or the environment variable MC_REFERENCE_DIR:

    python tests/golden/make_golden.py --ref PATH_TO_REFERENCE

For every case it writes a seeded synthetic click log (the package's
generator, reference text format), compiles the reference's CPU path out of
tree (oracle/ref/Makefile -> oracle/_ref/ref_driver), runs it with one thread,
and stores in <case>.npz:

  * the log itself (as text bytes) and the partition the reference built from
    it (train/test query ids, doc ids, click masks, parameter indices, n_qd);
  * every parameter (numerator, denominator; float32 bits) after selected
    iterations, in get_parameters(ALL) order;
  * the reference's test-set LogLikelihood / Perplexity sums and final values.

The fixtures pin the oracle (tests/test_oracle_golden.py) and the product's
ingest (tests/test_ingest.py).  Nothing reads the reference at test time.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from massiveclicks_gb300 import api  # noqa: E402
from massiveclicks_gb300 import build  # noqa: E402

DUMP_ITERS = (1, 2, 5, 10, 20)

# name, generator preset, sessions, queries, pool, model, iterations
SYNTH_CASES = [
    ("pbm_pbmclicks", 0, 4000, 150, 20, 0, 20),
    ("ubm_dbnclicks", 1, 4000, 200, 30, 3, 20),
    ("dbn_dbnclicks", 1, 4000, 200, 30, 2, 20),
    ("ccm_ccmclicks", 2, 4000, 200, 50, 1, 20),
    ("dbn_ccmclicks", 2, 4000, 200, 50, 2, 20),
]


def edge_log() -> str:
    """A small hand-made log with the corner cases the parser and the E-step
    meet: repeated clicks, clicks on docs not shown, duplicate docs in one
    result list, sessions with no clicks and with every rank clicked, lines of
    the wrong length and with a non-numeric session id, and a test tail with an
    unseen query, a session whose docs are all unseen and one partly seen."""
    lines = []
    sid = 0

    def q(query, docs, clicks=()):
        nonlocal sid
        lines.append(f"{sid} 0 Q {query} 0 " + " ".join(str(d) for d in docs))
        for k, d in enumerate(clicks):
            lines.append(f"{sid} {k + 1} C {d}")
        sid += 1

    base = list(range(1, 11))
    q(5, base, [3, 3, 99])                       # repeated click, click on an unshown doc
    lines.append("this line has five tokens")     # wrong length: reported, skipped
    q(5, base[::-1])                              # no clicks
    q(6, [1, 1, 2, 2, 3, 3, 4, 4, 5, 5], [2, 4])  # duplicate docs: first matching rank clicked
    q(7, list(range(11, 21)), list(range(11, 21)))  # every rank clicked
    lines.append("abc 0 Q 5 0 1 2 3 4 5 6 7 8 9 10")  # non-numeric session id: skipped
    q(5, base, [10])                              # last rank clicked
    q(6, [5, 4, 3, 2, 1, 6, 7, 8, 9, 10], [5, 6])
    q(7, list(range(20, 10, -1)), [19])
    q(5, [2, 1, 4, 3, 6, 5, 8, 7, 10, 9], [1, 2, 3])
    q(8, list(range(30, 40)), [30])
    q(6, [1, 2, 3, 4, 5, 11, 12, 13, 14, 15], [13])
    q(5, base, [1])
    q(7, list(range(11, 21)), [])
    q(8, list(range(35, 45)), [44])
    q(5, base, [2, 7])
    q(6, [2, 1, 2, 1, 3, 4, 5, 6, 7, 8], [1])
    # test tail
    q(99, base, [1])                              # unseen query: dropped
    q(5, list(range(100, 110)), [100])            # query seen, no doc seen: dropped
    q(8, [30, 31, 100, 101, 32, 33, 102, 34, 35, 36], [31])  # partly seen
    q(6, [1, 2, 3, 4, 5, 6, 7, 8, 9, 10], [])
    q(5, base, [])                                # trailing session: never kept by the reader
    return "\n".join(lines) + "\n"


def read_partition(d: Path) -> dict:
    out = {}
    for name in ("train", "test"):
        q = np.fromfile(d / f"{name}_query.i32", np.int32)
        out[f"{name}_query"] = q
        out[f"{name}_docs"] = np.fromfile(d / f"{name}_doc.i32", np.int32).reshape(-1, 10)
        out[f"{name}_pidx"] = np.fromfile(d / f"{name}_pidx.i32", np.int32).reshape(-1, 10)
        clicks = np.fromfile(d / f"{name}_click.u8", np.uint8).reshape(-1, 10)
        out[f"{name}_click"] = api.clicks_to_mask(clicks)
    n_train, n_test, n_qd = (int(x) for x in (d / "meta.txt").read_text().split())
    assert out["train_query"].shape[0] == n_train and out["test_query"].shape[0] == n_test
    out["n_qd"] = np.int64(n_qd)
    return out


def run_case(driver: Path, name: str, log_text: str, max_sessions: int, models, iters: int) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        log = tmp / "log.txt"
        log.write_text(log_text)
        data = {"log": np.frombuffer(log_text.encode(), np.uint8), "max_sessions": np.int64(max_sessions),
                "test_share": np.float32(0.2), "iterations": np.int64(iters), "models": np.array(models, np.int64)}
        for model in models:
            out = tmp / f"m{model}"
            out.mkdir()
            subprocess.run([str(driver), "em", str(log), str(max_sessions), "0.2", str(model), str(iters), "1",
                            str(out), "1"], check=True, stdout=subprocess.DEVNULL)
            part = read_partition(out)
            for k, v in part.items():
                if k in data:
                    assert np.array_equal(data[k], v), k
                data[k] = v
            for it in DUMP_ITERS:
                if it <= iters:
                    data[f"m{model}_params_{it:04d}"] = np.fromfile(out / f"params_{it:04d}.f32", np.float32).reshape(-1, 2)
            ev = {}
            for line in (out / "eval.txt").read_text().splitlines():
                key, val = line.split()
                ev[key] = float.fromhex(val) if "x" in val else float(val)
            data[f"m{model}_llh_sum"] = np.float64(ev["llh_sum"])
            data[f"m{model}_llh"] = np.float64(ev["llh"])
            data[f"m{model}_ppl"] = np.float64(ev["ppl"])
            data[f"m{model}_log2_sums"] = np.array([ev[f"log2sum_{r}"] for r in range(10)], np.float64)
            # The driver's loop must agree with the reference's own em_parallel,
            # which also writes its parameter CSVs (kept as text for the CLI test).
            prefix = out / "csv"
            res = subprocess.run([str(driver), "em_parallel", str(log), str(max_sessions), "0.2", str(model),
                                  str(iters), "1", str(prefix)], check=True, capture_output=True, text=True)
            for csv in sorted(out.glob("csv_*.csv")):
                data[f"m{model}_csv_{csv.stem[4:]}"] = np.frombuffer(csv.read_bytes(), np.uint8)
            llh_line = [x for x in res.stdout.splitlines() if x.startswith("Total Log likelihood is:")][0]
            em_llh = float(llh_line.split(":")[1])
            assert abs(em_llh - ev["llh"]) <= 1e-5 * abs(ev["llh"]), (em_llh, ev["llh"])
        np.savez_compressed(HERE / f"{name}.npz", **data)
        print(f"{name}: train {data['train_query'].shape[0]} test {data['test_query'].shape[0]} n_qd {int(data['n_qd'])}")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MC_REFERENCE_DIR"),
                    help="checkout of the reference's sources (default: $MC_REFERENCE_DIR)")
    args = ap.parse_args()
    if not args.ref:
        sys.exit("name the reference's source checkout with --ref or MC_REFERENCE_DIR")
    build.build_library()
    driver = build.build_reference(args.ref)
    if driver is None:
        sys.exit(f"reference sources not found at {args.ref}")
    for name, preset, n, nq, pool, model, iters in SYNTH_CASES:
        cfg = api.synth_config(preset, n_sessions=n, n_queries=nq, pool=pool)
        with tempfile.TemporaryDirectory() as tmp:
            path = Path(tmp) / "log.txt"
            api.write_log(cfg, str(path))
            text = path.read_text()
        run_case(driver, name, text, n, [model], iters)
    run_case(driver, "edge", edge_log(), 1000, [0, 1, 2, 3], 5)


if __name__ == "__main__":
    main()
