#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

The fixtures are outputs of the reference's own code, built from its sources
by oracle/Makefile (`make -C oracle ref`, outputs in oracle/_ref/):

* ``<test>.stdout.gz`` -- stdout of the reference's hand-written REF oracles
  ``tests/system_tests/test_cases/<test>.manual.ref.c``.  The reference's
  system-test driver diffs a translated program's stdout against exactly this
  text (tests/system_tests/run_system_tests.sh.cmake:833-883).
* ``diffusion_ref_n21_c6.*`` -- initial field, final field and coefficients
  of the reference's sequential clamped 7-point diffusion
  (examples/diffusion-benchmark/baseline.cc:22-49) on a 21^3 grid, 6 steps.
* ``himeno_ref_33x17x19_nn3.*`` -- p after 3 sweeps and the last sweep's gosa
  of the original Himeno jacobi (examples/himeno/himenobmtxpa_original.c:297-346)
  on rows=33 (Physis z), cols=17 (y), deps=19 (x).

``manifest.json`` records each file's SHA-256 and the parameters.  Run from
the repository root with the reference tree present:

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

MANUAL_TESTS = [
    "test_7-pt",
    "test_7-pt-neumann-cond",
    "test_7-pt-multi-iterations",
    "test_7-pt-double-type",
    "test_7-pt-int-type",
    "test_7-pt-periodic",
    "test_reduction-3d-sum",
    "test_3-pt-1d",
    "test_3-pt-periodic",
    "test_5-pt-2d",
    "test_5-pt-periodic",
    "test_9-pt-2d",
    "test_9-pt-reduction",
    "test_9-pt-periodic-reduction",
    "test_27-pt",
    "test_27-pt-periodic",
    "test_27-pt-reduction",
    "test_asymmetric",
    "test_asymmetric-periodic",
    "test_stencil-hole",
    "test_redblack",
    "test_redblack-periodic",
    "test_16",
    "test_15",
    "test_7-pt-type-mix",
    "test_mixed-dim",
    "test_mixed-dim2",
    "test_mixed-dim3",
    # grids of user-defined struct types
    "test_user-defined-type-7-pt",
    "test_user-defined-type-7-pt-periodic",
    "test_user-defined-type-7-pt-periodic-complex",
    "test_user-defined-type-multi-dim-member",
    "test_user-defined-type-multi-members",
    "test_user-defined-type1",
    "test_user-defined-type3",
    "test_user-defined-type5",
]

DIFF_N, DIFF_COUNT = 21, 6
HIM_ROWS, HIM_COLS, HIM_DEPS, HIM_NN = 33, 17, 19, 3


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def gz_write(path, data):
    # mtime=0 keeps the gzip bytes reproducible
    with open(path, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as f:
            f.write(data)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    if not os.path.isdir(args.ref):
        sys.exit(f"reference tree not found at {args.ref}")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"),
                           "ref", f"REF={args.ref}"])
    manifest = {"generator": "tests/golden/make_golden.py", "files": {}}

    for t in MANUAL_TESTS:
        exe = os.path.join(REF_DIR, f"{t}.manual.ref.exe")
        out = subprocess.run([exe], check=True, capture_output=True).stdout
        dst = os.path.join(HERE, f"{t}.stdout.gz")
        gz_write(dst, out)
        manifest["files"][os.path.basename(dst)] = {
            "source": f"tests/system_tests/test_cases/{t}.manual.ref.c",
            "stdout_sha256": hashlib.sha256(out).hexdigest(),
            "sha256": sha256(dst)}

    tmp = os.path.join(REF_DIR, "tmp_golden")
    os.makedirs(tmp, exist_ok=True)
    pre = os.path.join(tmp, "diff")
    subprocess.check_call([os.path.join(REF_DIR, "ref_diffusion_harness.exe"),
                           str(DIFF_N), str(DIFF_COUNT), pre])
    stem = f"diffusion_ref_n{DIFF_N}_c{DIFF_COUNT}"
    for suffix in ("init.f32", "final.f32"):
        with open(f"{pre}.{suffix}", "rb") as f:
            data = f.read()
        dst = os.path.join(HERE, f"{stem}.{suffix}.gz")
        gz_write(dst, data)
        manifest["files"][os.path.basename(dst)] = {
            "source": "examples/diffusion-benchmark/baseline.cc:22-49",
            "n": DIFF_N, "count": DIFF_COUNT, "sha256": sha256(dst)}
    dst = os.path.join(HERE, f"{stem}.coef.txt")
    shutil.copyfile(f"{pre}.coef.txt", dst)
    manifest["files"][os.path.basename(dst)] = {
        "order": "ce cw cn cs ct cb cc", "sha256": sha256(dst)}

    pre = os.path.join(tmp, "him")
    subprocess.check_call([os.path.join(REF_DIR, "ref_himeno_harness.exe"),
                           str(HIM_ROWS), str(HIM_COLS), str(HIM_DEPS),
                           str(HIM_NN), pre])
    stem = f"himeno_ref_{HIM_ROWS}x{HIM_COLS}x{HIM_DEPS}_nn{HIM_NN}"
    with open(f"{pre}.p.f32", "rb") as f:
        data = f.read()
    dst = os.path.join(HERE, f"{stem}.p.f32.gz")
    gz_write(dst, data)
    manifest["files"][os.path.basename(dst)] = {
        "source": "examples/himeno/himenobmtxpa_original.c:297-346",
        "rows_z": HIM_ROWS, "cols_y": HIM_COLS, "deps_x": HIM_DEPS,
        "nn": HIM_NN, "sha256": sha256(dst)}
    dst = os.path.join(HERE, f"{stem}.gosa.txt")
    shutil.copyfile(f"{pre}.gosa.txt", dst)
    manifest["files"][os.path.basename(dst)] = {"sha256": sha256(dst)}
    shutil.rmtree(tmp)

    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
        f.write("\n")
    print(f"wrote {len(manifest['files'])} fixtures to {HERE}")


if __name__ == "__main__":
    main()
