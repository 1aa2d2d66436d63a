"""Build recipe for oracle/_ref: the reference's own CUDA kernels as sm_103a cubins.

Test infrastructure only.  Runs where the reference sources exist
(/root/reference/st_spix/csrc/bist); outputs go to oracle/_ref/ only:

  * <unit>.cubin        device code of the reference translation units that hold the
                        kernels of the bist_forward path, compiled from the sources
                        where they lie, unmodified, with -fmad=false (the same
                        no-contraction rule as the engine and the oracle) and -DNDEBUG;
  * stock/<unit>.cubin  the same units with nvcc's default contraction (FP32/FP64
                        multiply-adds fused, as the reference's own setup.py builds
                        them: setup.py:106-108 passes only -w --extended-lambda);
  * spix_layout.h       byte offsets of the reference's spix_params fields, printed by
  * spix_layout.json    a small program compiled against the reference's structs.h,
                        plus the sizes and the decision fields of its helper structs.

Build shims only: an empty opencv2/core/core.hpp, -include cstdint, the CUDA cccl path,
--extended-lambda (thrust lambdas in compact_spix.cu).  -DNDEBUG removes the device
asserts, so no reference kernel traps.  A cubin is device code, independent of the
host architecture, so the harness (oracle/ref_harness.cpp, built on the GPU host) loads
it through the CUDA driver API and launches the reference kernels on identical inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("STSPIX_REFERENCE", "/root/reference")
BIST = os.path.join(REF, "st_spix", "csrc", "bist")
# Translation units whose kernels bist_forward launches (setup.py:79-101 lists them).
UNITS = ["update_seg", "seg_utils", "update_params", "init_seg", "split_merge",
         "fill_missing", "split_disconnected", "rgb2lab", "split_merge_orig",
         "split_merge_prop", "relabel", "shift_labels", "sp_pooling", "init_sparams",
         "sparams_io", "compact_spix"]
VARIANTS = {"": ["-fmad=false"], "stock": []}
FIELDS = ["mu_app", "prior_mu_app", "mu_shape", "sigma_shape", "prior_mu_shape",
          "prior_sigma_shape", "sample_sigma_shape", "prior_icov", "logdet_sigma_shape",
          "count", "icount", "prior_count", "valid", "prop", "sm_count",
          "prior_mu_app_count", "prior_mu_shape_count", "prior_sigma_shape_count",
          "logdet_prior_sigma_shape", "prior_lprob"]
HELPER_FIELDS = ["sum_app", "sq_sum_app", "sum_shape", "sq_sum_shape"]
SM_FIELDS = ["sum_app", "sq_sum_app", "sum_shape", "count", "count_f", "hasting", "merge",
             "remove", "select"]
SM2_FIELDS = ["sum_app", "sq_sum_app", "sum_shape", "count", "ninvalid", "hasting", "merge",
              "remove", "select"]


def available() -> bool:
    return os.path.isfile(os.path.join(BIST, "update_seg.cu"))


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _compile(cmd, verbose):
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)


def build(force: bool = False, verbose: bool = False) -> bool:
    if not available():
        return False
    os.makedirs(os.path.join(OUT, "stubs", "opencv2", "core"), exist_ok=True)
    open(os.path.join(OUT, "stubs", "opencv2", "core", "core.hpp"), "w").close()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    common = ["-gencode", "arch=compute_103a,code=sm_103a", "-DNDEBUG", "-w",
              "--extended-lambda", "-I" + os.path.join(cuda_inc, "cccl"), "-include",
              "cstdint", "-I" + os.path.join(OUT, "stubs")]
    jobs = []
    for sub, flags in VARIANTS.items():
        d = os.path.join(OUT, sub)
        os.makedirs(d, exist_ok=True)
        for u in UNITS:
            out = os.path.join(d, u + ".cubin")
            src = os.path.join(BIST, u + ".cu")
            if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
                continue
            jobs.append([nvcc(), "-cubin", *common, *flags, "-o", out, src])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_compile, j, verbose) for j in jobs]:
            f.result()
    # struct layouts
    prog = os.path.join(OUT, "layout_probe.cu")
    lines = ['#include "structs.h"', "#include <cstdio>", "#include <cstddef>",
             "int main(){",
             '  printf("#define REF_SP_SIZE %zu\\n", sizeof(spix_params));',
             '  printf("#define REF_HELPER_SIZE %zu\\n", sizeof(spix_helper));',
             '  printf("#define REF_SM_SIZE %zu\\n", sizeof(spix_helper_sm));',
             '  printf("#define REF_SM2_SIZE %zu\\n", sizeof(spix_helper_sm_v2));']
    for f in FIELDS:
        lines.append(f'  printf("#define REF_OFF_{f} %zu\\n", offsetof(spix_params, {f}));')
    for f in HELPER_FIELDS:
        lines.append(f'  printf("#define REF_HOFF_{f} %zu\\n", offsetof(spix_helper, {f}));')
    for f in SM_FIELDS:
        lines.append(f'  printf("#define REF_SMOFF_{f} %zu\\n", offsetof(spix_helper_sm, {f}));')
    for f in SM2_FIELDS:
        lines.append(f'  printf("#define REF_SM2OFF_{f} %zu\\n", '
                     f'offsetof(spix_helper_sm_v2, {f}));')
    lines.append("  return 0; }")
    open(prog, "w").write("\n".join(lines) + "\n")
    exe = os.path.join(OUT, "layout_probe")
    subprocess.run([nvcc(), "-w", "-I" + BIST, "-I" + os.path.join(cuda_inc, "cccl"), "-o", exe,
                    prog], check=True)
    layout = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    open(os.path.join(OUT, "spix_layout.h"), "w").write(
        "// generated by oracle/ref_build.py from the reference's structs.h\n" + layout)
    table = {}
    for line in layout.splitlines():
        _, name, val = line.split()
        table[name] = int(val)
    with open(os.path.join(OUT, "spix_layout.json"), "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv, verbose=True)
    print("built oracle/_ref" if ok else "reference sources not present: nothing built")
