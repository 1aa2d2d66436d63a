"""Build recipe for oracle/_ref: the reference's own CUDA kernels as sm_103a cubins.

Test infrastructure only.  Runs where the reference sources exist
(/root/reference/st_spix/csrc/bist); outputs go to oracle/_ref/ only:

  * <file>.cubin        device code of selected reference translation units, compiled
                        from the sources where they lie, unmodified, with
                        -fmad=false (the same no-contraction rule as the engine and
                        the oracle) and -DNDEBUG; build shims only: an empty
                        opencv2/core/core.hpp, -include cstdint, the CUDA cccl path;
  * spix_layout.h       byte offsets of the reference's spix_params fields, printed by
                        a small program compiled against the reference's structs.h.

A cubin is device code, independent of the host architecture, so the harness
(oracle/ref_harness.cpp, built on the GPU host) can load it through the CUDA driver
API and launch the reference kernels on identical inputs.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("STSPIX_REFERENCE", "/root/reference")
BIST = os.path.join(REF, "st_spix", "csrc", "bist")
UNITS = ["update_seg", "seg_utils", "update_params", "init_seg", "split_merge",
         "fill_missing", "split_disconnected", "rgb2lab"]
FIELDS = ["mu_app", "prior_mu_app", "mu_shape", "sigma_shape", "prior_mu_shape",
          "prior_sigma_shape", "sample_sigma_shape", "prior_icov", "logdet_sigma_shape",
          "count", "icount", "prior_count", "valid", "prop"]


def available() -> bool:
    return os.path.isfile(os.path.join(BIST, "update_seg.cu"))


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build(force: bool = False, verbose: bool = False) -> bool:
    if not available():
        return False
    os.makedirs(os.path.join(OUT, "stubs", "opencv2", "core"), exist_ok=True)
    open(os.path.join(OUT, "stubs", "opencv2", "core", "core.hpp"), "w").close()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    common = ["-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false", "-DNDEBUG", "-w",
              "-I" + os.path.join(cuda_inc, "cccl"), "-include", "cstdint",
              "-I" + os.path.join(OUT, "stubs")]
    for u in UNITS:
        out = os.path.join(OUT, u + ".cubin")
        src = os.path.join(BIST, u + ".cu")
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        cmd = [nvcc(), "-cubin", *common, "-o", out, src]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    # spix_params layout
    prog = os.path.join(OUT, "layout_probe.cu")
    lines = ['#include "structs.h"', "#include <cstdio>", "#include <cstddef>",
             "int main(){",
             '  printf("#define REF_SP_SIZE %zu\\n", sizeof(spix_params));']
    for f in FIELDS:
        lines.append(f'  printf("#define REF_OFF_{f} %zu\\n", offsetof(spix_params, {f}));')
    lines.append("  return 0; }")
    open(prog, "w").write("\n".join(lines) + "\n")
    exe = os.path.join(OUT, "layout_probe")
    subprocess.run([nvcc(), "-w", "-I" + BIST, "-I" + os.path.join(cuda_inc, "cccl"), "-o", exe,
                    prog], check=True)
    layout = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    open(os.path.join(OUT, "spix_layout.h"), "w").write(
        "// generated by oracle/ref_build.py from the reference's structs.h\n" + layout)
    return True


if __name__ == "__main__":
    ok = build(force="--force" in sys.argv, verbose=True)
    print("built oracle/_ref" if ok else "reference sources not present: nothing built")
