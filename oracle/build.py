"""Test-oracle only: build recipes for the CPU oracle.

* `build_oracle()` compiles the restatement oracle/hodlr_oracle.cpp into
  oracle/liboracle.so (g++, OpenMP, -ffp-contract=off so that every scalar
  operation rounds once, as the parity tests assume).
* `build_ref(ndim, nmax, dprime, eps)` compiles the reference's own headers,
  in place under the reference checkout, with oracle/ref_config.hpp standing in
  for the hand-edited include/myHeaders.hpp and oracle/eigen_min for Eigen,
  into oracle/_ref/ref_driver_<tag>.  Nothing from the reference is copied;
  the binaries stay out of version control.  When the reference checkout is
  absent (it only exists where the fixtures are generated) this returns None.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("HODLRND_REFERENCE", "/root/reference")
REF_INCLUDE = os.path.join(REF_ROOT, "include")
OUT_REF = os.path.join(HERE, "_ref")


def build_oracle(force=False):
    src = os.path.join(HERE, "hodlr_oracle.cpp")
    out = os.path.join(HERE, "liboracle.so")
    stamp = os.path.join(HERE, "liboracle.machine")
    if not os.path.exists(stamp) or open(stamp).read() != platform.machine():
        force = True
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-Wall", src, "-o", out]
    subprocess.run(cmd, check=True)
    with open(stamp, "w") as f:
        f.write(platform.machine())
    return out


def ref_tag(ndim, nmax, dprime, eps, user_kernels=False):
    t = f"d{ndim}_n{nmax}_p{dprime}_e{eps:.0e}".replace("-", "m").replace("+", "")
    return t + ("_uk" if user_kernels else "")


def build_ref(ndim, nmax, dprime, eps, user_kernels=False, force=False):
    if not os.path.isdir(REF_INCLUDE):
        return None
    os.makedirs(OUT_REF, exist_ok=True)
    out = os.path.join(OUT_REF, "ref_driver_" + ref_tag(ndim, nmax, dprime, eps, user_kernels))
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_config.hpp")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-w", "-DUSE_DOUBLE",
           f"-DREF_NDIM={ndim}", f"-DREF_NMAX={nmax}", f"-DREF_DPRIME={dprime}", f"-DREF_EPS={eps!r}",
           "-include", os.path.join(HERE, "ref_config.hpp"),
           "-I" + HERE, "-I" + os.path.join(HERE, "eigen_min"), "-I" + REF_INCLUDE]
    if user_kernels:
        cmd.append("-DREF_WITH_USER_KERNELS")
    cmd += [os.path.join(HERE, "ref_driver.cpp"), "-o", out]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
