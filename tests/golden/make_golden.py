"""Generate the golden fixtures from the reference PLSQR3 program itself.

Runs only where the reference tree is mounted (it builds oracle/_ref/PLSQR3
from the reference's own sources with `make -C oracle ref`).  For each case
the synthetic inputs are written in the reference's file formats, the
reference program is run on them (one rank, FP64 build), and its outputs are
stored here:

  <case>/x.f64           p_resultx_itn=<K>_NProc=1_float64_mpiio.bin (small
                         cases; the large ones keep its sha256 in meta.json)
  <case>/result.txt      the reference's Paige-Saunders log
  <case>/alpha_beta.txt  alpha_k, beta_k at %.17e (k = 0..K)
  <case>/meta.json       iterations, file names, sha256 of every input file,
                         sha256 of the in-memory arrays (array_digest)
  tiny/inputs/*          the input files themselves (small case only)

The large cases (the 96x96x32 grid with 20,000 and 200,000 rays) also run the
oracle on the same arrays, check that its x, alpha_k and beta_k equal the
reference's bit for bit, and store its per-iteration scalars:

  <case>/hist.txt        k rnorm arnorm anorm xnorm test1 test2 at %.17e

so that a GPU test can hold every iteration of the big solve against the
reference without running a CPU solve of its own.

The large cases also get ulp.txt: how far the reference's own scalars move
when every element of b_k is raised by one ulp (see ulp_sensitivity).

tests/golden/socal25 comes from the reference's own data/ sample (its first
25 rays; see run_socal).

Usage: python tests/golden/make_golden.py [case ...]   (default: tiny grid32)
       cases: tiny grid32 grid96s grid96 socal25 grid32p
       python tests/golden/make_golden.py --ulp case ...  (ulp.txt only)
The 200,000-ray case writes 21 GB of input files to the temporary directory
and takes about an hour on 8 cores (the reference's kernel-row product is
single-threaded).
"""
from __future__ import annotations

import gc
import hashlib
import json
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import __graft_entry__ as g  # noqa: E402

# name -> (commit the input files too, store the oracle's per-iteration scalars)
CASES = {"tiny": (True, False), "grid32": (False, False),
         "grid96s": (False, True), "grid96": (False, True)}
HIST_KEYS = ("rnorm", "arnorm", "anorm", "xnorm", "test1", "test2")
INPUT_KEYS = ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k")


def sha256(p: Path) -> str:
    h = hashlib.sha256()
    with open(p, "rb") as f:
        while True:
            chunk = f.read(1 << 24)
            if not chunk:
                break
            h.update(chunk)
    return h.hexdigest()


def array_digest(prob) -> str:
    """sha256 over the arrays of a generated problem, in a fixed order: the
    kernel by column, the damping matrix by row and by column (ptr as int64,
    idx as int32, val as float64) and b_k.  Cheaper than writing the files."""
    h = hashlib.sha256()
    for lines in (prob.k_csc, prob.d_csr, prob.d_csc):
        for a, dt in ((lines.ptr, np.int64), (lines.idx, np.int32), (lines.val, np.float64)):
            h.update(memoryview(np.ascontiguousarray(a, dt)).cast("B"))
    h.update(memoryview(np.ascontiguousarray(prob.b_k, np.float64)).cast("B"))
    return h.hexdigest()


def run_case(name: str, pkg, orc, ref: Path) -> None:
    keep_inputs, with_hist = CASES[name]
    out = HERE / name
    it = pkg.CONFIGS[name]["iterations"]
    t0 = time.time()
    prob = pkg.generate(name)
    digest = array_digest(prob)
    nnz_k, nnz_d = prob.meta["nnz_k"], prob.meta["nnz_d"]
    print(f"{name}: generated nnz_k={nnz_k} in {time.time() - t0:.0f} s", flush=True)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        files = pkg.write_files(prob, td / "in")
        hist = None
        if with_hist:
            t0 = time.time()
            o = orc.OracleProblem(prob).lsqr(it)
            hist, ox = o["hist"], o["x"]
            print(f"{name}: oracle {it} iterations in {time.time() - t0:.0f} s", flush=True)
        del prob
        gc.collect()
        run = td / "run"
        run.mkdir()
        cmd = [str(ref), "-dir", str(td / "in")]
        for k in INPUT_KEYS:
            cmd += [f"-{k}", files[k]]
        cmd += ["-row_k", str(files["row_k"]), "-row_d", str(files["row_d"]),
                "-col", str(files["col"]), "-itn", str(it)]
        t0 = time.time()
        r = subprocess.run(cmd, cwd=run, capture_output=True, text=True, check=True)
        print(f"{name}: reference {it} iterations in {time.time() - t0:.0f} s", flush=True)
        lines = r.stdout.splitlines()
        al = [l.split()[1] for l in lines if l.startswith("ORACLE_alpha")]
        be = [l.split()[1] for l in lines if l.startswith("ORACLE_beta")]
        assert len(al) == len(be) == it + 1, (len(al), len(be))
        x = np.fromfile(run / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", np.float64)
        if hist is not None:
            # the stored scalars are the oracle's: valid only if its run is the
            # reference's run, bit for bit
            assert np.array_equal(ox, x), "oracle x differs from the reference"
            assert np.array_equal(hist["alpha"], np.array([float(a) for a in al]))
            assert np.array_equal(hist["beta"], np.array([float(b) for b in be]))
        if out.exists():
            shutil.rmtree(out)
        out.mkdir()
        x.tofile(out / "x.f64")
        shutil.copy(run / "result.txt", out / "result.txt")
        (out / "alpha_beta.txt").write_text(
            "".join(f"{k} {a} {b}\n" for k, (a, b) in enumerate(zip(al, be))))
        if hist is not None:
            (out / "hist.txt").write_text(
                "# k " + " ".join(HIST_KEYS) + "\n"
                + "".join(f"{k} " + " ".join(f"{hist[key][k]:.17e}" for key in HIST_KEYS) + "\n"
                          for k in range(it + 1)))
        sums = {files[k]: sha256(td / "in" / files[k]) for k in INPUT_KEYS}
        meta = dict(case=name, iterations=it, files={k: v for k, v in files.items() if k != "dir"}
                    | {"dir": "inputs"}, sha256=sums, array_sha256=digest, nnz_k=nnz_k,
                    nnz_d=nnz_d,
                    reference_time=[l for l in lines if "Parallel LSQR time" in l])
        (out / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
        if keep_inputs:
            shutil.copytree(td / "in", out / "inputs")
    print(f"{name}: {it} iterations, nnz_k={nnz_k}, written to {out}", flush=True)


def ulp_sensitivity(name: str, pkg, orc) -> None:
    """How far the reference's own per-iteration scalars move when every
    element of b_k is raised by one ulp (a change of the size of the
    rounding differences between two summation orders; one element alone is
    absorbed by the rounding of the first norm and product on the 200,000-ray
    problem): the oracle (bitwise equal to the reference) is run on the
    perturbed b and compared with the stored golden run.  Written to
    <case>/ulp.txt (k, then the relative change of alpha, beta, rnorm,
    arnorm) and, while x.f64 is still there (right after the golden run),
    meta.json["ulp_x_rel"] (the change of x), after which x.f64 is replaced by
    its digest.  The reference tree is not needed."""
    out = HERE / name
    meta = json.loads((out / "meta.json").read_text())
    it = meta["iterations"]
    prob = pkg.generate(name)
    assert array_digest(prob) == meta["array_sha256"]
    b = np.nextafter(prob.b_k, np.inf)
    t0 = time.time()
    o = orc.OracleProblem(prob).lsqr(it, b_k=b)
    print(f"{name}: perturbed oracle run in {time.time() - t0:.0f} s", flush=True)
    ab = np.loadtxt(out / "alpha_beta.txt")
    hist = np.loadtxt(out / "hist.txt")
    rel = lambda a, r: np.abs(a - r) / np.maximum(np.abs(r), 1e-300)
    cols = [rel(o["hist"]["alpha"], ab[:, 1]), rel(o["hist"]["beta"], ab[:, 2]),
            rel(o["hist"]["rnorm"], hist[:, 1]), rel(o["hist"]["arnorm"], hist[:, 2])]
    (out / "ulp.txt").write_text(
        "# relative change of the reference's scalars when every element of b_k is raised "
        "by one ulp\n# k alpha beta rnorm arnorm\n"
        + "".join(f"{k} " + " ".join(f"{c[k]:.3e}" for c in cols) + "\n" for k in range(it + 1)))
    xf = out / "x.f64"
    meta.pop("ulp_x_rel", None)
    if xf.exists():
        x = np.fromfile(xf, np.float64)
        meta["ulp_x_rel"] = float(np.linalg.norm(o["x"] - x) / np.linalg.norm(x))
        # the large cases keep the digest of x, not x (2.4 MB): a GPU test
        # holds its reference-order x to the digest and its other x to that one
        meta["x_sha256"] = hashlib.sha256(x.tobytes()).hexdigest()
        xf.unlink()
    (out / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")


# ---- the reference's data/ sample (SoCal): its first SOCAL_RAYS rays ----------
SOCAL_RAYS = 25
SOCAL_ITN = 100  # data/LSQR_run/LSQR3.pbs:10


def reference_data_dir(orc) -> Path:
    return orc.REF_SRC.parent / "data"


def convert_with_reference_tools(orc, data: Path, names: list[str], ncol: int,
                                 work: Path) -> Path:
    """The reference's own kernel-format tools on the ray files `names`:
    ker_ascii2bin, Ker2PLSQR3_preprocess, Ker2PLSQR3 (compiled by
    `make -C oracle tools`).  Returns the directory holding their
    matrix_bycol.mm2.bin / .info."""
    subprocess.run(["make", "-s", "-C", str(orc.HERE), "tools", f"REF_SRC={orc.REF_SRC}"],
                   check=True)
    tools = orc.HERE / "_ref"
    bins = work / "ker_bin"
    bins.mkdir(parents=True, exist_ok=True)
    (work / "ker.list").write_text(f"{len(names)}\n" + "".join(f"{nm}\n" for nm in names))
    subprocess.run([str(tools / "ker_ascii2bin"), str(work / "ker.list"),
                    str(data / "ker_ASCII"), str(bins)], check=True, capture_output=True)
    counts = [sum(1 for ln in open(data / "ker_ASCII" / nm) if ln.split()) for nm in names]
    (bins / "ker_bin.list").write_text("".join(f"{nm}.bin {c}\n" for nm, c in zip(names, counts)))
    subprocess.run([str(tools / "Ker2PLSQR3_preprocess"), str(bins), "ker_bin.list", str(ncol)],
                   check=True, capture_output=True)
    subprocess.run([str(tools / "Ker2PLSQR3"), str(bins), "ker_bin.list", str(ncol),
                    str(bins / "col_info.txt")], check=True, capture_output=True)
    return bins


def run_socal(pkg, orc, ref: Path, n_rays: int = SOCAL_RAYS) -> None:
    """tests/golden/socal<n>: the first n rays of the reference's data/ sample
    with the damping matrix of its README (every weight 1.0, 2 fields).  The
    kernel files are made by the reference's own tools and must equal the
    restated conversion byte for byte; the reference program then runs
    SOCAL_ITN iterations on them, and the oracle must reproduce its bits.
    Stored: rays.npz (the rays in raykernels' lossless compact form and
    b_k), alpha_beta.txt, hist.txt, result.txt, meta.json with the sha256 of
    x (x itself is 2.4 MB: a GPU test compares its own x's digest)."""
    R = pkg.raykernels
    data = reference_data_dir(orc)
    name = f"socal{n_rays}"
    out = HERE / name
    names = R.read_list(data / "ker.list")[:n_rays]
    rays = [R.read_ascii_ray(data / "ker_ASCII" / nm) for nm in names]
    b = np.loadtxt(data / "measure_fake.list")[:n_rays]
    prob = R.socal_from_rays(rays, b)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        files = pkg.write_files(prob, td / "in")
        tool_dir = convert_with_reference_tools(orc, data, names, prob.n, td / "tools")
        for k, fn in (("ker_f", "matrix_bycol.mm2.bin"), ("ker_i", "matrix_bycol.mm2.info")):
            assert (td / "in" / files[k]).read_bytes() == (tool_dir / fn).read_bytes(), \
                f"{fn} differs from the reference tools' output"
        o = orc.OracleProblem(prob).lsqr(SOCAL_ITN)
        run = td / "run"
        run.mkdir()
        cmd = [str(ref), "-dir", str(td / "in")]
        for k in INPUT_KEYS:
            cmd += [f"-{k}", files[k]]
        cmd += ["-row_k", str(prob.m_k), "-row_d", str(prob.m_d), "-col", str(prob.n),
                "-itn", str(SOCAL_ITN)]
        r = subprocess.run(cmd, cwd=run, capture_output=True, text=True, check=True)
        lines = r.stdout.splitlines()
        al = [l.split()[1] for l in lines if l.startswith("ORACLE_alpha")]
        be = [l.split()[1] for l in lines if l.startswith("ORACLE_beta")]
        assert len(al) == len(be) == SOCAL_ITN + 1
        x = np.fromfile(run / f"p_resultx_itn={SOCAL_ITN}_NProc=1_float64_mpiio.bin", np.float64)
        assert np.array_equal(o["x"], x), "oracle x differs from the reference"
        assert np.array_equal(o["hist"]["alpha"], np.array([float(a) for a in al]))
        assert np.array_equal(o["hist"]["beta"], np.array([float(v) for v in be]))
        if out.exists():
            shutil.rmtree(out)
        out.mkdir()
        np.savez_compressed(out / "rays.npz", b_k=b, **R.socal_compact(rays))
        shutil.copy(run / "result.txt", out / "result.txt")
        (out / "alpha_beta.txt").write_text(
            "".join(f"{k} {a} {v}\n" for k, (a, v) in enumerate(zip(al, be))))
        hist = o["hist"]
        (out / "hist.txt").write_text(
            "# k " + " ".join(HIST_KEYS) + "\n"
            + "".join(f"{k} " + " ".join(f"{hist[key][k]:.17e}" for key in HIST_KEYS) + "\n"
                      for k in range(SOCAL_ITN + 1)))
        meta = dict(case=name, iterations=SOCAL_ITN, n_rays=n_rays, m_k=prob.m_k, m_d=prob.m_d,
                    n=prob.n, nnz_k=prob.meta["nnz_k"], nnz_d=prob.meta["nnz_d"],
                    array_sha256=array_digest(prob),
                    x_sha256=hashlib.sha256(x.tobytes()).hexdigest(),
                    kernel_files_sha256={files[k]: sha256(td / "in" / files[k])
                                         for k in ("ker_f", "ker_i")},
                    rays=names, reference_time=[l for l in lines if "Parallel LSQR time" in l])
        (out / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print(f"{name}: {SOCAL_ITN} iterations, nnz_k={prob.meta['nnz_k']}, written to {out}",
          flush=True)


# ---- the column permutation of the COL_PERM build ------------------------------
PERM_SEED = 2013


def run_col_perm(pkg, orc, ref: Path, base: str = "grid32") -> None:
    """tests/golden/<base>p: the reference's solve of <base> with its kernel
    columns permuted as the COL_PERM build loads them (column i = file column
    perm[i], damping and b as given, x in the permuted order).  That build
    itself cannot run: source/plsqr3.c:283 frees the column info array and
    sets it to NULL, and :328-329 hand the NULL to the reordered loader,
    which dereferences it (:1698).  Its loader is a pure selection of
    columns, so the reference program is run on the kernel file written with
    the columns already permuted: the matrix that loader would build.  The
    permutation is numpy's PCG64 permutation of seed PERM_SEED."""
    name = base + "p"
    out = HERE / name
    it = pkg.CONFIGS[base]["iterations"]
    prob = pkg.generate(base)
    perm = np.random.default_rng(PERM_SEED).permutation(prob.n).astype(np.int32)
    kp = pkg.synth.permute_columns(prob.k_csc, perm)
    permuted = pkg.Problem(kp, prob.d_csr, prob.d_csc, prob.b_k, prob.x_true, it, prob.meta)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        files = pkg.write_files(permuted, td / "in")
        pkg.synth.write_col_perm(td / "colPerm", perm)
        run = td / "run"
        run.mkdir()
        cmd = [str(ref), "-dir", str(td / "in")]
        for k in INPUT_KEYS:
            cmd += [f"-{k}", files[k]]
        cmd += ["-row_k", str(prob.m_k), "-row_d", str(prob.m_d), "-col", str(prob.n),
                "-itn", str(it)]
        r = subprocess.run(cmd, cwd=run, capture_output=True, text=True, check=True)
        lines = r.stdout.splitlines()
        al = [l.split()[1] for l in lines if l.startswith("ORACLE_alpha")]
        be = [l.split()[1] for l in lines if l.startswith("ORACLE_beta")]
        assert len(al) == len(be) == it + 1
        if out.exists():
            shutil.rmtree(out)
        out.mkdir()
        shutil.copy(run / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", out / "x.f64")
        shutil.copy(run / "result.txt", out / "result.txt")
        (out / "alpha_beta.txt").write_text(
            "".join(f"{k} {a} {b}\n" for k, (a, b) in enumerate(zip(al, be))))
        meta = dict(case=name, base=base, iterations=it, perm_seed=PERM_SEED,
                    col_perm_sha256=sha256(td / "colPerm"),
                    permuted_kernel_sha256={files[k]: sha256(td / "in" / files[k])
                                            for k in ("ker_f", "ker_i")},
                    files={k: v for k, v in files.items() if k != "dir"} | {"dir": "inputs"},
                    reference_time=[l for l in lines if "Parallel LSQR time" in l])
        (out / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print(f"{name}: {it} iterations with permuted columns, written to {out}", flush=True)


def main(names) -> None:
    pkg = g.load_package()
    orc = g.load_oracle()
    if names and names[0] == "--ulp":
        for name in names[1:]:
            ulp_sensitivity(name, pkg, orc)
        return
    orc.build(with_reference=True)
    ref = orc.REF_BIN
    if not ref.exists():
        raise SystemExit("reference program not built (is the reference tree mounted?)")
    for name in names:
        if name.startswith("socal"):
            run_socal(pkg, orc, ref, int(name[5:] or SOCAL_RAYS))
            continue
        if name.endswith("p") and name[:-1] in CASES:
            run_col_perm(pkg, orc, ref, name[:-1])
            continue
        run_case(name, pkg, orc, ref)
        if CASES[name][1]:
            ulp_sensitivity(name, pkg, orc)


if __name__ == "__main__":
    main(sys.argv[1:] or ["tiny", "grid32"])
