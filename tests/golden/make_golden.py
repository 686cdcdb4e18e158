"""Regenerate the golden fixtures from the reference tree (run in a checkout that has it).

Reads the reference's committed C-atom example (examples/C: FCIDUMP, config.json, result.json,
the run log `out`) and its unit-test constants, and writes:
  c_atom/FCIDUMP, c_atom/config.json  - the example's inputs, copied verbatim
  c_atom_pins.json                    - numbers parsed from the example's log and result.json
From the Cr-dimer example (examples/Cr, point group D-infinity-h) it writes:
  cr_dimer/FCIDUMP.gz, cr_dimer/config.json - the inputs (the FCIDUMP gzip-compressed)
  cr_dimer_pins.json                  - HF energy, queue size, and per variational iteration
                                        the det count, nnz, energy and Davidson trace, up to
                                        the first eps_var's first iteration (see the note in
                                        the pins file on the later ones)
The Davidson Hilbert-matrix known answers (src/solver/davidson_test.cc:5-51) and the
HalfDet unit-test cases (src/det/half_det_test.cc:30-46) are transcribed into hilbert_pins.json
and halfdet_pins.json by reading those files as text.

Usage: python tests/golden/make_golden.py [/path/to/reference]
(default: $SHCI_REFERENCE, else /root/reference)
"""
import gzip
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_int(s):
    return int(s.replace(",", ""))


def main(ref):
    ex = os.path.join(ref, "examples", "C")
    os.makedirs(os.path.join(HERE, "c_atom"), exist_ok=True)
    for f in ("FCIDUMP", "config.json"):
        shutil.copyfile(os.path.join(ex, f), os.path.join(HERE, "c_atom", f))
    out = open(os.path.join(ex, "out")).read().splitlines()
    pins = {"source": "examples/C (out, result.json)"}
    m = next(l for l in out if l.startswith("HF energy:"))
    pins["energy_hf"] = float(m.split()[2])
    pins["max_hci_queue_elem"] = float(
        next(l for l in out if l.startswith("Max hci queue elem")).split()[4])
    pins["n_hci_queue_entries"] = parse_int(
        next(l for l in out if l.startswith("Number of entries in hci queue")).split()[-1])
    pins["max_singles_queue_elem"] = float(
        next(l for l in out if l.startswith("Max singles_queue elem")).split()[3])
    pins["n_singles_queue_entries"] = parse_int(
        next(l for l in out if l.startswith("Number of entries in singles_queue")).split()[-1])
    # Per variational iteration: dets after selection, nnz (symmetric count), energy.
    iters = []
    cur = {}
    for l in out:
        m = re.match(r"Number of dets / new dets: ([\d,]+) / ([\d,]+)", l)
        if m:
            cur = {"n_dets": parse_int(m.group(1)), "n_new": parse_int(m.group(2))}
        m = re.match(r"Number of nonzero elems: ([\d,]+)", l)
        if m:
            cur["nnz"] = parse_int(m.group(1))
        m = re.match(r"Iteration (\d+) eps1= (\S+) ndets= ([\d,]+) energy= (\S+)", l)
        if m:
            cur.update(iteration=int(m.group(1)), eps1=float(m.group(2)),
                       ndets=parse_int(m.group(3)), energy=float(m.group(4)))
            iters.append(cur)
            cur = {}
    pins["iterations"] = iters
    res = json.load(open(os.path.join(ex, "result.json")))
    pins["energy_var"] = res["energy_var"]
    pins["energy_total"] = {k: v for k, v in res["energy_total"].items() if k != "extrapolated"}
    # Deterministic PT stage lines.
    dtm = []
    for i, l in enumerate(out):
        m = re.match(r"PT dtm correction \(eps1= (\S+), eps_pt_dtm= (\S+)\): (\S+)", l)
        if m:
            nl = [x for x in out[max(0, i - 4):i] if x.startswith("Number of dtm pt dets")]
            dtm.append({"eps_var": float(m.group(1)), "eps_pt_dtm": float(m.group(2)),
                        "correction": float(m.group(3)),
                        "n_pt_dets": parse_int(nl[-1].split()[-1]) if nl else None})
    pins["pt_dtm"] = dtm
    # First pseudo-stochastic batch of each eps_var (the log's batch count is 16).
    psto = []
    for i, l in enumerate(out):
        m = re.match(r"PT psto correction \(eps1= (\S+), eps_pt_psto= (\S+)\): (\S+) \+- (\S+)", l)
        if m:
            head = out[max(0, i - 12):i]
            if not any(x.startswith("BEG OF #1/") for x in head):
                continue
            nl = [x for x in head if x.startswith("Number of psto pt dets")]
            nb = [x for x in out[max(0, i - 30):i] if x.startswith("Number of psto batches")]
            psto.append({"eps_var": float(m.group(1)), "eps_pt_psto": float(m.group(2)),
                         "correction": float(m.group(3)), "uncert": float(m.group(4)),
                         "n_pt_dets": parse_int(nl[-1].split()[-1]),
                         "n_batches": int(nb[-1].split()[-1])})
    pins["pt_psto_first_batch"] = psto
    json.dump(pins, open(os.path.join(HERE, "c_atom_pins.json"), "w"), indent=1)

    dt = open(os.path.join(ref, "src", "solver", "davidson_test.cc")).read()
    vals = re.search(r"expected_eigenvalues\(\s*\{([^}]*)\}", dt).group(1)
    vecs = re.search(r"expected_eigenvectors\(\s*\{\{([^}]*)\}", dt).group(1)
    hil = {"source": "src/solver/davidson_test.cc", "n": 1000, "gamma": 10.0,
           "eigenvalue0": float(vals.split(",")[0]),
           "eigenvector0_head": [float(x) for x in vecs.split(",")],
           "tol_value": 1e-6, "tol_vector": 1e-4, "davidson_tol": 1e-6}
    json.dump(hil, open(os.path.join(HERE, "hilbert_pins.json"), "w"), indent=1)

    hd = open(os.path.join(ref, "src", "det", "half_det_test.cc")).read()
    assert "EXPECT_EQ(diff.right_only[0], 3)" in hd
    halfdet = {"source": "src/det/half_det_test.cc:30-46",
               "cases": [{"a": [0], "b": [1], "n_diffs": 1, "left0": 0, "right0": 1},
                         {"a": [0, 1], "b": [1, 3], "n_diffs": 1, "left0": 0, "right0": 3}]}
    json.dump(halfdet, open(os.path.join(HERE, "halfdet_pins.json"), "w"), indent=1)
    cr_dimer(ref)
    print("wrote golden fixtures to", HERE)


def cr_dimer(ref):
    ex = os.path.join(ref, "examples", "Cr")
    dst = os.path.join(HERE, "cr_dimer")
    os.makedirs(dst, exist_ok=True)
    shutil.copyfile(os.path.join(ex, "config.json"), os.path.join(dst, "config.json"))
    with open(os.path.join(ex, "FCIDUMP"), "rb") as f, \
            gzip.GzipFile(os.path.join(dst, "FCIDUMP.gz"), "wb", 9, mtime=0) as g:
        g.write(f.read())
    out = open(os.path.join(ex, "out")).read().splitlines()
    cfg = json.load(open(os.path.join(ex, "config.json")))
    pins = {"source": "examples/Cr (out, config.json)",
            "n_up": cfg["n_up"], "n_dn": cfg["n_dn"],
            "point_group": cfg["chem"]["point_group"],
            "eps_vars": cfg["eps_vars"], "eps_vars_schedule": cfg["eps_vars_schedule"],
            "target_error": cfg["target_error"],
            "note": "The log was written by an older build than the reference source: it has "
                    "no singles-queue lines, and from the second iteration at one eps_var on "
                    "(iteration 6) its selection finds fewer dets than the current source "
                    "does. The pins stop before that iteration."}
    pins["energy_hf"] = float(next(l for l in out if l.startswith("HF energy:")).split()[2])
    pins["max_hci_queue_elem"] = float(
        next(l for l in out if l.startswith("Max hci queue elem")).split()[4])
    pins["n_hci_queue_entries"] = parse_int(
        next(l for l in out if l.startswith("Number of entries in hci queue")).split()[-1])
    iters, cur, trace = [], {}, []
    for l in out:
        m = re.match(r"Number of dets / new dets: ([\d,]+) / ([\d,]+)", l)
        if m:
            cur = {"n_dets": parse_int(m.group(1)), "n_new": parse_int(m.group(2))}
            trace = []
        m = re.match(r"Number of nonzero elems: ([\d,]+)", l)
        if m:
            cur["nnz"] = parse_int(m.group(1))
        m = re.match(r"Davidson #(\d+): (\S+)", l)
        if m:
            trace.append(float(m.group(2)))
        m = re.match(r"Iteration (\d+) eps1= (\S+) ndets= ([\d,]+) energy= (\S+)", l)
        if m:
            cur.update(iteration=int(m.group(1)), eps1=float(m.group(2)),
                       ndets=parse_int(m.group(3)), energy=float(m.group(4)),
                       davidson=trace)
            iters.append(cur)
            cur = {}
    # up to and including the first iteration at the first eps_var
    first = next(k for k, it in enumerate(iters) if it["eps1"] == cfg["eps_vars"][0])
    pins["iterations"] = iters[:first + 1]
    json.dump(pins, open(os.path.join(HERE, "cr_dimer_pins.json"), "w"), indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1
         else os.environ.get("SHCI_REFERENCE", "/root/reference"))
