"""Recipe: compile the Correlator_node adapter (sfxc-1_gb300/adapter/) against
the REFERENCE's own headers and link it with the reference's compiled classes
and libsfxc_gpu.so -- the check that the drop-in builds where a maintainer
would put it.

Test infrastructure only.  Uses the objects oracle/build_ref.py compiles from
the reference checkout (Time, Data_writer, Correlation_parameters' types) and
its shims (config.h, the MPI stand-in, sfxc_abort), with the reference's
flags (-O2 -ffast-math -std=gnu++03).  Output: oracle/_ref/adapter_main.
Returns None when the reference checkout is absent.
"""
import os
import subprocess

from . import build_ref

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
MAIN = os.path.join(ROOT, "tests", "adapter_main.cc")
ADAPTER = os.path.join(ROOT, "sfxc-1_gb300", "adapter", "correlator_node_gpu.h")
LIBDIR = os.path.join(ROOT, "sfxc-1_gb300", "lib")


def exe_path():
    return os.path.join(build_ref.OUT, "adapter_main")


def build(ref_root=None, force=False):
    ref_root = ref_root or build_ref.default_root()
    if build_ref.build(ref_root) is None:
        return None
    sfxc = os.path.join(ref_root, "sfxc")
    exe = exe_path()
    lib = os.path.join(LIBDIR, "libsfxc_gpu.so")
    deps = [MAIN, ADAPTER, lib, os.path.join(ROOT, "include", "sfxc_gpu.h")]
    if os.path.exists(exe) and not force and os.path.getmtime(exe) >= max(os.path.getmtime(f) for f in deps):
        return exe
    out = build_ref.OUT
    incs = ["-I" + os.path.join(out, "inc"), "-I" + build_ref.SHIM, "-I" + os.path.join(sfxc, "include"),
            "-I" + os.path.join(sfxc, "src"), "-I" + os.path.join(sfxc, "lib/common/src"),
            "-I" + os.path.join(sfxc, "lib/containers/src"), "-I" + os.path.join(sfxc, "lib/jsoncpp/include"),
            "-I" + os.path.join(sfxc, "lib/vex_parser/vex_parser/include"), "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.dirname(ADAPTER)]
    obj = os.path.join(out, "obj")
    objs = sorted(os.path.join(obj, f) for f in os.listdir(obj) if f.endswith(".o") and f != "harness.o")
    main_o = os.path.join(out, "adapter_main.o")
    cmd = ["g++", "-std=gnu++03", "-O2", "-ffast-math", "-DBOOST_SP_USE_PTHREADS", "-Wall", "-Wno-unused",
           "-ffunction-sections", "-fdata-sections"] + incs + ["-c", MAIN, "-o", main_o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter compile failed:\n%s%s" % (r.stdout, r.stderr))
    tmp = exe + ".tmp%d" % os.getpid()
    link = ["g++", "-o", tmp, main_o] + objs + ["-Wl,--gc-sections", "-L" + LIBDIR, "-lsfxc_gpu",
                                                 "-Wl,-rpath," + LIBDIR, "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, exe)
    return exe


if __name__ == "__main__":
    print(build(force=True) or "reference checkout absent; nothing built")
