"""Generate the golden fixtures from the reference PLSQR3 program itself.

Runs only where the reference tree is mounted (it builds oracle/_ref/PLSQR3
from the reference's own sources with `make -C oracle ref`).  For each case
the synthetic inputs are written in the reference's file formats, the
reference program is run on them (one rank, FP64 build), and its outputs are
stored here:

  <case>/x.f64         p_resultx_itn=<K>_NProc=1_float64_mpiio.bin
  <case>/result.txt    the reference's Paige-Saunders log
  <case>/alpha_beta.txt  alpha_k, beta_k at %.17e (k = 0..K)
  <case>/inputs.sha256   sha256 of every input file
  tiny/inputs/*        the input files themselves (small case only)

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as g  # noqa: E402

CASES = {"tiny": True, "grid32": False}  # name -> commit the inputs too


def sha256(p: Path) -> str:
    return hashlib.sha256(p.read_bytes()).hexdigest()


def main() -> None:
    pkg = g.load_package()
    orc = g.load_oracle()
    orc.build(with_reference=True)
    ref = orc.REF_BIN
    if not ref.exists():
        raise SystemExit("reference program not built (is the reference tree mounted?)")
    for name, keep_inputs in CASES.items():
        out = HERE / name
        if out.exists():
            shutil.rmtree(out)
        out.mkdir()
        prob = pkg.generate(name)
        it = pkg.CONFIGS[name]["iterations"]
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            files = pkg.write_files(prob, td / "in")
            run = td / "run"
            run.mkdir()
            cmd = [str(ref), "-dir", str(td / "in")]
            for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
                cmd += [f"-{k}", files[k]]
            cmd += ["-row_k", str(prob.m_k), "-row_d", str(prob.m_d), "-col", str(prob.n),
                    "-itn", str(it)]
            r = subprocess.run(cmd, cwd=run, capture_output=True, text=True, check=True)
            shutil.copy(run / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", out / "x.f64")
            shutil.copy(run / "result.txt", out / "result.txt")
            lines = r.stdout.splitlines()
            al = [l.split()[1] for l in lines if l.startswith("ORACLE_alpha")]
            be = [l.split()[1] for l in lines if l.startswith("ORACLE_beta")]
            assert len(al) == len(be) == it + 1, (len(al), len(be))
            (out / "alpha_beta.txt").write_text(
                "".join(f"{k} {a} {b}\n" for k, (a, b) in enumerate(zip(al, be))))
            sums = {files[k]: sha256(td / "in" / files[k])
                    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol",
                              "damp_i_bycol", "b_k")}
            meta = dict(case=name, iterations=it, files=files | {"dir": "inputs"}, sha256=sums,
                        nnz_k=prob.meta["nnz_k"], nnz_d=prob.meta["nnz_d"],
                        reference_time=[l for l in lines if "Parallel LSQR time" in l])
            (out / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
            if keep_inputs:
                shutil.copytree(td / "in", out / "inputs")
        print(f"{name}: {it} iterations, nnz_k={prob.meta['nnz_k']}, written to {out}")


if __name__ == "__main__":
    main()
