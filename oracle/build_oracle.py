"""Build the C restatement checker (oracle/sfxc_oracle.c) into oracle/_build/.

Test infrastructure only.  Compiled without fast-math and without FP
contraction so that its float and double operations round exactly where the
source says.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "sfxc_oracle.c")


def exe_path():
    return os.path.join(OUT, "sfxc_oracle")


def build(force=False):
    exe = exe_path()
    if not force and os.path.exists(exe) and os.path.getmtime(exe) >= os.path.getmtime(SRC):
        return exe
    os.makedirs(OUT, exist_ok=True)
    tmp = exe + ".tmp%d" % os.getpid()
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-o", tmp, SRC, "-lm"],
                   check=True, capture_output=True, text=True)
    os.replace(tmp, exe)
    return exe


if __name__ == "__main__":
    print(build(force=True))
