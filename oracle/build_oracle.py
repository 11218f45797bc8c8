"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` — the project's CPU restatement of the
  reference hot path (oracle/sph_oracle.cpp).  Built everywhere.
* ``oracle/_ref/libsphref.so`` — the reference's own CPU path compiled
  unmodified from ``src/sph.cpp``, ``src/neighborTable.cpp`` and
  ``src/timer.cpp`` of the reference checkout, against the project-written
  GLM shim in ``oracle/shim``, plus oracle/ref_harness.cpp.  Built only where
  the reference checkout exists (``SPH_REFERENCE_DIR``, default
  ``/root/reference``); elsewhere the restatement alone is available.

Both use ``-O2 -ffp-contract=off -pthread`` (the reference's CMakeLists sets
no optimisation level; contraction is disabled so that no multiply-add is
fused on either x86-64 or aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FLAGS = ["-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-pthread", "-w"]
REF_SOURCES = ["sph.cpp", "neighborTable.cpp", "timer.cpp"]


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in inputs)


def build_port(force=False):
    out = os.path.join(HERE, "_build", "liboracle.so")
    src = os.path.join(HERE, "sph_oracle.cpp")
    if force or _stale(out, [src]):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call(["g++", *FLAGS, src, "-o", out])
    return out


def reference_dir():
    return os.environ.get("SPH_REFERENCE_DIR", "/root/reference")


def build_ref(force=False):
    """Returns the path of libsphref.so, or None where the reference is absent."""
    src_dir = os.path.join(reference_dir(), "src")
    if not os.path.isfile(os.path.join(src_dir, "sph.cpp")):
        return None
    out = os.path.join(HERE, "_ref", "libsphref.so")
    harness = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "shim")
    srcs = [os.path.join(src_dir, s) for s in REF_SOURCES] + [harness]
    deps = srcs + [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    if force or _stale(out, deps):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call(["g++", *FLAGS, "-I", shim, "-I", src_dir, *srcs, "-o", out])
    return out


def main():
    force = "--force" in sys.argv
    print(build_port(force))
    print(build_ref(force))


if __name__ == "__main__":
    main()
