"""Recipe: compile the REFERENCE's correlator-node classes into a CPU checker.

Test infrastructure only.  It compiles, directly with g++/gcc, the reference's
own source files for the correlator-node hot path where they lie under the
reference checkout, plus the GSL 1.9 interpolation sources from the tarball the
reference vendors (sfxc/lib/gsl/gsl-1.9.tar.gz), and links them with
oracle/ref_harness.cc and the shims in oracle/ref_shim/ (config.h, an FFTW3
API over a double-precision FFT, an in-process MPI stand-in, and the VEX grammar restated in
vex_grammar.cc because flex and bison are absent).  Every output
goes to oracle/_ref/ (git-ignored).  The reference's own build system is not
used.

Flags follow the reference (sfxc/configure.ac:31,98-101): -O2 -ffast-math
-std=gnu++03.  -DBOOST_SP_USE_PTHREADS makes the vendored boost shared_ptr
portable (sfxc/include/boost/detail/sp_counted_base.hpp:26-60).

Usage:  python oracle/build_ref.py [reference_root]
The reference root defaults to the REF_ROOT environment variable, else a
checkout named `reference` beside the repository's own directory.  Returns
without building when the checkout is absent.
"""
import os
import shutil
import subprocess
import sys
import tarfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def default_root():
    """REF_ROOT, else the `reference` checkout beside the repository."""
    return os.environ.get("REF_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
SHIM = os.path.join(HERE, "ref_shim")

REF_SOURCES = [
    "src/bit2float_worker.cc",
    "src/bit_statistics.cc",
    "src/delay_correction.cc",
    "src/correlation_core.cc",
    "src/correlation_core_pulsar.cc",
    "src/correlation_core_phased.cc",
    "src/delay_table_akima.cc",
    "src/correlator_time.cc",
    "src/sfxc_fft_float.cc",
    "src/data_writer.cc",
    "src/input_node_data_writer.cc",
    "src/input_node_tasklet.cc",
    "src/channel_extractor_5.cc",
    "src/control_parameters.cc",
    "src/vdif_reader.cc",
    "src/mark5b_reader.cc",
    "src/input_data_format_reader.cc",
    "src/input_data_format_reader_tasklet.cc",
    "src/mark5a_reader.cc",
    "src/uvw_model.cc",
    "src/data_reader.cc",
    "src/data_reader_file.cc",
    "src/data_reader_blocking.cc",
    "src/tasklet/tasklet.cc",
    "lib/common/src/align_malloc.cc",
    "lib/common/src/thread.cc",
    "lib/common/src/mutex.cc",
    "lib/common/src/condition.cc",
    "lib/common/src/raiimutex.cc",
    "lib/common/src/exception_common.cc",
    "lib/common/src/backtrace.cc",
    "lib/common/src/demangler.cc",
    "lib/containers/src/default_allocator.cc",
    "lib/vex_parser/vex_parser/src/Vexpp_node.cc",
    "lib/vex_parser/vex_parser/src/Vex++.cc",
    "lib/jsoncpp/src/json_reader.cpp",
    "lib/jsoncpp/src/json_value.cpp",
    "lib/jsoncpp/src/json_writer.cpp",
]
GSL_SOURCES = [
    "interpolation/accel.c",
    "interpolation/akima.c",
    "interpolation/bsearch.c",
    "interpolation/interp.c",
    "interpolation/spline.c",
    "err/error.c",
    "err/stream.c",
    "err/strerror.c",
    "err/message.c",
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def harness_path():
    return os.path.join(OUT, "ref_harness")


def build(ref_root=None, force=False):
    ref_root = ref_root or default_root()
    sfxc = os.path.join(ref_root, "sfxc")
    if not os.path.isdir(sfxc):
        return None
    exe = harness_path()
    # rebuild when the harness or the shims changed since the last build
    own = [os.path.join(HERE, "ref_harness.cc")] + [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
    if os.path.exists(exe) and not force and os.path.getmtime(exe) >= max(os.path.getmtime(f) for f in own):
        return exe
    obj = os.path.join(OUT, "obj")
    inc = os.path.join(OUT, "inc")
    os.makedirs(obj, exist_ok=True)
    os.makedirs(os.path.join(inc, "gsl"), exist_ok=True)
    # types.h includes "../config.h": with -I<OUT>/inc it resolves to <OUT>/config.h
    shutil.copy(os.path.join(SHIM, "config.h"), os.path.join(OUT, "config.h"))

    gsl_dir = os.path.join(OUT, "gsl-1.9")
    if not os.path.isdir(gsl_dir):
        with tarfile.open(os.path.join(sfxc, "lib/gsl/gsl-1.9.tar.gz")) as t:
            members = [m for m in t.getmembers()
                       if m.name.startswith(("gsl-1.9/interpolation/", "gsl-1.9/err/"))
                       or (m.name.startswith("gsl-1.9/") and m.name.endswith(".h"))]
            t.extractall(OUT, members=members)
    for root, _, files in os.walk(gsl_dir):
        for f in files:
            if f.startswith("gsl_") and f.endswith(".h"):
                shutil.copy(os.path.join(root, f), os.path.join(inc, "gsl", f))
    gslcfg = os.path.join(OUT, "gslcfg")
    os.makedirs(gslcfg, exist_ok=True)
    with open(os.path.join(gslcfg, "config.h"), "w") as f:
        f.write("/* GSL built with its defaults (macros normally from its configure) */\n"
                "#define DISCARD_POINTER(p) do { ; } while (p ? 0 : 0);\n"
                "#define RETURN_IF_NULL(x) if (!x) { return ; }\n")

    incs = ["-I" + inc, "-I" + SHIM,
            "-I" + os.path.join(sfxc, "include"), "-I" + os.path.join(sfxc, "src"),
            "-I" + os.path.join(sfxc, "lib/common/src"),
            "-I" + os.path.join(sfxc, "lib/containers/src"),
            "-I" + os.path.join(sfxc, "lib/testunit/src"),
            "-I" + os.path.join(sfxc, "lib/jsoncpp/include"),
            "-I" + os.path.join(sfxc, "lib/vex_parser/vex_parser/include")]
    cxx = ["g++", "-std=gnu++03", "-O2", "-ffast-math", "-DBOOST_SP_USE_PTHREADS",
           "-ffunction-sections", "-fdata-sections", "-w"] + incs
    jobs = []
    for s in REF_SOURCES:
        o = os.path.join(obj, "ref_" + s.replace("/", "_") + ".o")
        jobs.append(cxx + ["-c", os.path.join(sfxc, s), "-o", o])
    for s in GSL_SOURCES:
        o = os.path.join(obj, "gsl_" + s.replace("/", "_") + ".o")
        jobs.append(["gcc", "-O2", "-std=gnu89", "-w", "-ffunction-sections", "-fdata-sections",
                     "-I" + gslcfg, "-I" + inc, "-I" + os.path.join(gsl_dir, "interpolation"),
                     "-c", os.path.join(gsl_dir, s), "-o", o])
    for s in ["fftw_shim.cc", "sfxc_stubs.cc"]:
        jobs.append(["g++", "-O2", "-I" + SHIM, "-ffunction-sections", "-fdata-sections",
                     "-c", os.path.join(SHIM, s), "-o", os.path.join(obj, "shim_" + s + ".o")])
    # the VEX grammar, restated (no flex/bison here), over the reference's Vexpp_node
    jobs.append(cxx + ["-I" + os.path.join(sfxc, "lib/vex_parser/vex_parser/src"),
                       "-c", os.path.join(SHIM, "vex_grammar.cc"), "-o", os.path.join(obj, "shim_vex_grammar.o")])
    jobs.append(cxx + ["-c", os.path.join(HERE, "ref_harness.cc"),
                       "-o", os.path.join(obj, "harness.o")])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    objs = sorted(os.path.join(obj, f) for f in os.listdir(obj) if f.endswith(".o"))
    _run(["g++", "-o", exe] + objs + ["-Wl,--gc-sections", "-lpthread"])
    return exe


def build_output_header(ref_root=None):
    """oracle/ref_output_header.cc against the reference's output_header.h:
    prints the bytes of a filled Output_header_global.  None without the checkout."""
    ref_root = ref_root or default_root()
    inc = os.path.join(ref_root, "sfxc", "include")
    if not os.path.isfile(os.path.join(inc, "output_header.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_output_header")
    src = os.path.join(HERE, "ref_output_header.cc")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        _run(["g++", "-O2", "-std=gnu++03", "-I" + inc, src, "-o", exe])
    return exe


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None, force=True)
    print(path or "reference checkout absent; nothing built")
