"""Log of the engine-versus-reference comparisons made by the parity tests.

Every logged comparison is one JSON line: the workload, the step (initial
partition, iteration k, run), whether the labels are identical, and the WCC of
both sides with its relative difference (the engine sums the WCC terms in a
fixed tree order, the reference in index order, so the last bits may differ;
labels may not).  Lines go to the file named by the SCD_PARITY_LOG environment
variable when it is set; the session summary (tests/conftest.py) reports the
number of comparisons, of label divergences and of WCC values whose bits differ.
"""
import json
import os

RECORDS = []


def log(workload, step, **fields):
    rec = {"workload": workload, "step": step, **fields}
    if "wcc" in rec and "wcc_ref" in rec:
        rec["wcc_bits_equal"] = rec["wcc"] == rec["wcc_ref"]
    RECORDS.append(rec)
    path = os.environ.get("SCD_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")


def summary():
    if not RECORDS:
        return None
    div = sum(1 for r in RECORDS if r.get("labels_equal") is False)
    bits = sum(1 for r in RECORDS if r.get("wcc_bits_equal") is False)
    worst = max((r.get("wcc_rel", 0.0) for r in RECORDS), default=0.0)
    return (f"parity log: {len(RECORDS)} comparisons, {div} label divergences, "
            f"{bits} WCC values differing in the last bits (largest relative difference {worst:.3g})")
