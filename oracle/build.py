"""Build the oracle (test infrastructure): the C restatement ``cbc_oracle.c`` into
``oracle/libcbc_oracle.so`` and, when the reference checkout is present, the reference's
own CPU module into ``oracle/_ref/`` (``build_ref.sh``).  Neither is product code."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libcbc_oracle.so")


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "cbc_oracle.c"), os.path.join(HERE, "oracle_impl.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(s) for s in src):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", src[0], "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_reference() -> None:
    """the reference's CPU module (compiled here), and its GPU module's sources staged
    into oracle/_ref/cuda_src for a build on the GPU host (oracle/ref_cuda.py); both
    are no-ops without the reference checkout"""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.run(["bash", script], check=True)
    subprocess.run(["bash", os.path.join(HERE, "build_ref_cuda.sh"), "stage"], check=True)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    build_reference()
