"""ORACLE recipe -- builds oracle/_ref/ from the DYFOX reference sources.

Test infrastructure only.  DYFOX keeps its three Laue kernels as CUDA text
inside ``laue/kernels.py`` (lines 48-352) and instantiates them for FP32 or
FP64 with its own ``kernels.build`` (lines 19-44, 361-369), which hands the
text to CuPy.  This script imports the reference read-only (no bytecode is
written), replaces ``backend.cupy`` by a stub whose ``RawKernel`` records
the text, and writes the six instantiations, each renamed with a
``_f64``/``_f32`` suffix and wrapped in a namespace of its own, its
``extern __shared__`` buffer renamed by a macro so that the float and double
declarations do not collide, to:

    oracle/_ref/ref_kernels.inc     the kernel text, verbatim otherwise
    oracle/_ref/ref_cpu.cpp         includes ref_cpu_shim.h + the text (g++)
    oracle/_ref/ref_gpu.cu          includes the text + ref_launch_gpu.cuh
                                    (nvcc, for the GPU parity tests)

``oracle/_ref`` is git-ignored; the generated text travels with the tree so
that ``build()`` can compile it on a machine without the reference.  Run:

    python oracle/make_ref.py [--reference PATH]
"""

import argparse
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def extract(reference):
    sys.dont_write_bytecode = True
    sys.path.insert(0, reference)
    import backend                                    # noqa: E402

    captured = {}

    class RawKernel:                                  # CuPy stand-in
        def __init__(self, src, name):
            captured[name] = src

    stub = types.SimpleNamespace(RawKernel=RawKernel)
    backend.cupy = lambda: stub
    from laue import kernels                          # noqa: E402
    kernels.cupy = lambda: stub
    texts = []
    for prec in (backend.FP64, backend.FP32):
        suffix = "_f32" if prec.is_fp32 else "_f64"
        for name in ("fullfield", "analytic", "pristine"):
            captured.clear()
            kernels.build(name, prec)
            (fname, src), = captured.items()
            real = "float" if prec.is_fp32 else "double"
            ns = f"ref_{name}{suffix}"
            # The block-scope `extern __shared__ T smem[]` of a kernel with
            # C linkage is itself a C-linkage name: give each instantiation
            # its own so the float and double declarations do not collide.
            texts.append(f"#define smem {ns}_smem\n"
                         f"namespace {ns} {{\n"
                         + src.replace(fname + "(", fname + suffix + "(")
                         + f"\n}}  // namespace {ns}\n"
                         f"REF_SMEM_DEF({real}, {ns}_smem)\n"
                         "#undef smem\n#undef PI\n")
    sys.path.remove(reference)
    return "\n".join(texts)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    if not os.path.isdir(os.path.join(args.reference, "laue")):
        print(f"no reference at {args.reference}; nothing generated")
        return 1
    os.makedirs(OUT, exist_ok=True)
    text = extract(args.reference)
    with open(os.path.join(OUT, "ref_kernels.inc"), "w") as f:
        f.write("/* generated by oracle/make_ref.py from DYFOX "
                "laue/kernels.py -- do not commit */\n" + text)
    with open(os.path.join(OUT, "ref_cpu.cpp"), "w") as f:
        f.write('#include "../ref_cpu_shim.h"\n#include "ref_kernels.inc"\n'
                '#include "../ref_launch_cpu.inc"\n')
    with open(os.path.join(OUT, "ref_gpu.cu"), "w") as f:
        f.write('#define REF_SMEM_DEF(T, NAME)\n#include "ref_kernels.inc"\n'
                '#include "../ref_launch_gpu.cuh"\n')
    print(f"wrote {OUT}/ref_kernels.inc ({len(text)} bytes)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
