#!/usr/bin/env python3
"""Generate the full-size fixtures in tests/golden/full/ by running the
upstream FCFC on the benchmark workloads at their stated sizes.

The upstream executables are compiled from their own sources by
``make -f oracle/Makefile.ref REF=<FCFC checkout>`` (scalar FP64 + OpenMP)
into oracle/_ref/.  The catalogues are too large to commit: each one is
named by a ``synth.catalogue`` spec (generator, sizes, seeds) and the sha256
of its bytes, which the tests regenerate and check before they compare
counts.  What is committed per case directory:
  meta.json                 the catalogue specs and hashes, and per run the
                            FCFC configuration (bins, pairs, estimator)
  <run>_<PAIR>.bin          FCFC's binary pair-count file
  <run>_mp.txt / _wp.txt    FCFC's multipoles and w_p (and one xi file)

Cases (the benchmark configurations):
  c0_box_uniform   1e5 uniform points, L = 1000, DD (s, mu) 40 x 100, s < 200
  c1_box_ns        the Neyman-Scott box (2e4 parents, Poisson(100), sigma 5,
                   L = 2000, lognormal(0, 0.3) weights): (s, mu) 40 x 100 and
                   (s_perp, pi) 40 log s_perp in [0.1, 100) x 40 pi in [0, 40),
                   weighted and unweighted
  c1_box_ns_f32    the same catalogue rounded to float32
  c2_survey_ls     1e5 data / 3e5 randoms of the survey generator, RA/Dec/z
                   converted by FCFC (flat LCDM, Omega_m = 0.31), FKP weights;
                   DD, DR, RR in (s, mu) 40 x 100 (weighted and unweighted)
                   and (s_perp, pi) with w_p (weighted)
  c3_mocks         the first nine mocks of the batched workload: eight that
                   FCFC accepts and one it rejects (s_max >= L / 2)

Usage: FCFC_REF_BIN=<dir with FCFC_2PT_BOX, FCFC_2PT> \
       python tests/golden/make_golden_full.py [case ...]
(default directory: oracle/_ref)
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from fcfc_gb300 import synth  # noqa: E402
from make_golden import write_conf  # noqa: E402

REF = os.environ.get("FCFC_REF_BIN", os.path.join(ROOT, "oracle", "_ref"))
OUT = os.path.join(HERE, "full")
NTHREAD = str(os.cpu_count() or 4)

SMU = dict(bintype=1, sbin=dict(smin=0, smax=200, ds=5), nmu=100)
LOG_SP = np.geomspace(0.1, 100.0, 41)
SPI = dict(bintype=2, sfile=np.c_[LOG_SP[:-1], LOG_SP[1:]],
           pbin=dict(pmin=0, pmax=40, dpi=1))
LS = "(DD - 2*DR + RR) / RR"


def cases():
    c = {}
    c["c0_box_uniform"] = dict(
        geometry="box",
        cats={"D": {"gen": "uniform_box", "n": 100000, "box": 1000.0,
                    "seed": 0}},
        runs=[dict(name="smu", box=[1000.0], pairs=["DD"], weighted=False,
                   cf=["DD / @@ - 1"], poles=[0, 2, 4], **SMU)])
    for name, f32 in (("c1_box_ns", False), ("c1_box_ns_f32", True)):
        spec = {"gen": "neyman_scott", "nparent": 20000, "box": 2000.0,
                "seed": 1, "weights": 0.3, "wseed": 2}
        if f32:
            spec["float32"] = True
        runs = [dict(name="smu_wt", weighted=True, poles=[0, 2, 4], **SMU),
                dict(name="smu", weighted=False, poles=[0, 2, 4], **SMU),
                dict(name="spi_wt", weighted=True, wp=True, **SPI),
                dict(name="spi", weighted=False, wp=True, **SPI)]
        for r in runs:
            r.update(box=[2000.0], pairs=["DD"], cf=["DD / @@ - 1"])
        c[name] = dict(geometry="box", cats={"D": spec}, runs=runs)
    dspec = {"gen": "survey", "n": 100000, "seed": 11}
    rspec = {"gen": "survey", "n": 300000, "seed": 12}
    c["c2_survey_ls"] = dict(
        geometry="survey",
        cats={"D": dict(dspec, weights="fkp"),
              "R": dict(rspec, weights="fkp", fkp_of=dspec)},
        runs=[dict(name="smu_wt", weighted=True, poles=[0, 2, 4], **SMU),
              dict(name="smu", weighted=False, poles=[0, 2, 4], **SMU),
              dict(name="spi_wt", weighted=True, wp=True, **SPI)],
        convert=True, omega_m=0.31)
    for r in c["c2_survey_ls"]["runs"]:
        r.update(pairs=["DD", "DR", "RR"], cf=[LS])
    _, boxes = synth.mock_boxes(9, seed=7, sizes_only=True)
    mocks = {}
    runs = []
    for j, L in enumerate(boxes):
        lab = "M%d" % j
        mocks[lab] = {"gen": "mock", "index": j, "seed": 7}
        runs.append(dict(name="m%d" % j, labels=[lab], box=[L], pairs=["DD"],
                         weighted=False, cf=["DD / @@ - 1"], poles=[0, 2, 4],
                         **SMU))
    c["c3_mocks"] = dict(geometry="box", cats=mocks, runs=runs)
    return c


def run_case(name, case):
    out = os.path.join(OUT, name)
    if os.path.isdir(out):
        shutil.rmtree(out)
    os.makedirs(out)
    box = case["geometry"] == "box"
    exe = os.path.join(REF, "FCFC_2PT_BOX" if box else "FCFC_2PT")
    arrays = {}
    meta = {"geometry": case["geometry"], "build": os.path.basename(exe),
            "cats": {}, "runs": []}
    for lab, spec in case["cats"].items():
        a = synth.catalogue(spec)
        arrays[lab] = a
        meta["cats"][lab] = {"spec": spec, "n": int(len(a)),
                             "sha256": synth.catalogue_sha256(a)}
    if case.get("convert"):
        meta.update(convert=True, omega_m=case["omega_m"])
    for run in case["runs"]:
        labels = run.get("labels") or list(case["cats"])
        sub = {}
        for lab in labels:
            a = arrays[lab]
            # FCFC's labels are single capitals: a mock counts as "D"
            sub[lab if len(lab) == 1 else "D"] = a if run["weighted"] else a[:, :3]
        rc = dict(run, cats=sub)
        if case.get("convert"):
            rc.update(convert=True, omega_m=case["omega_m"])
        t0 = time.time()
        with tempfile.TemporaryDirectory() as tmp:
            lines = write_conf(rc, tmp, box) + ["OUTPUT_FORMAT = 0"]
            conf = os.path.join(tmp, "run.conf")
            with open(conf, "w") as f:
                f.write("\n".join(lines) + "\n")
            env = dict(os.environ, OMP_NUM_THREADS=NTHREAD)
            p = subprocess.run([exe, "-c", conf], env=env, capture_output=True,
                               text=True)
            m = {k: v for k, v in run.items() if k not in ("sfile",)}
            m["labels"] = labels
            if p.returncode != 0:
                # FCFC refuses the configuration (e.g. s_max >= L / 2)
                err = [l for l in (p.stdout + p.stderr).splitlines()
                       if "Error" in l or "error" in l]
                m["fcfc_rejected"] = True
                msg = err[0] if err else p.stderr
                m["fcfc_message"] = re.sub(r"\x1b\[[0-9;]*m", "", msg).strip()
            else:
                for pr in run["pairs"]:
                    shutil.copy(os.path.join(tmp, pr + ".bin"),
                                os.path.join(out, "%s_%s.bin" % (run["name"], pr)))
                # xi files are large at 40 x 100 bins: one case keeps them
                keep = ("mp.txt", "wp.txt") + (("xi.txt",) if name.startswith("c0")
                                               else ())
                for fn in keep:
                    if os.path.exists(os.path.join(tmp, fn)):
                        shutil.copy(os.path.join(tmp, fn),
                                    os.path.join(out, "%s_%s" % (run["name"], fn)))
            if "sfile" in run and not os.path.exists(os.path.join(out, "sbins.txt")):
                shutil.copy(os.path.join(tmp, "sbins.txt"),
                            os.path.join(out, "sbins.txt"))
            if "sfile" in run:
                m["sfile"] = "sbins.txt"
        m["fcfc_seconds"] = round(time.time() - t0, 2)
        meta["runs"].append(m)
        print("  %s/%s: %.1f s%s" % (name, run["name"], time.time() - t0,
                                     " (rejected)" if m.get("fcfc_rejected") else ""),
              flush=True)
    meta["threads"] = int(NTHREAD)
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", name, flush=True)


def main(argv):
    allc = cases()
    for n in (argv or sorted(allc)):
        run_case(n, allc[n])


if __name__ == "__main__":
    main(sys.argv[1:])
