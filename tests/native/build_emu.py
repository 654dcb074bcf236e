"""TEST INFRASTRUCTURE ONLY — builds tests/native/libtraverse_emu.so (host build of the BVH
builder, the shared traversal core and the shared principled BSDF) with g++ and -ffp-contract=off."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(REPO, "hiprt-path-tracer_gb300", "csrc")
LIB = os.path.join(HERE, "libtraverse_emu.so")
SRCS = [os.path.join(HERE, "traverse_emu.cpp"), os.path.join(HERE, "bsdf_emu.cpp"), os.path.join(CSRC, "bvh_build.cpp")]
DEPS = SRCS + [os.path.join(CSRC, n) for n in ("bvh.h", "trace_core.h", "principled.h", "hd_math.h")]


def build() -> str:
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-I", CSRC, "-I", os.path.join(REPO, "include"),
           "-o", LIB + ".tmp"] + SRCS
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build())
