"""Build recipe of oracle/_ref/: the reference's own CPU-path sources,
compiled where they lie in the reference checkout (never copied), against
self-written stand-ins for the headers they need and do not ship:

  * libref_hls.so  -- kernel/src/tfhe_blindRotate_FFT/{tGswFFTExternMulToTLwe,
    pease_fft, TorusPolynomial_fft, tLweFromFFTConvert, tfhe_MuxRotate_FFT,
    tfhe_blindRotate_FFT, tGswTorus32PolynomialDecompH, IntPolynomial_ifft,
    tLweFFTAddMulRTo}.cpp,
    tfhe_bootstrap_woKS_FFT/tfhe_bootstrap_woKS_FFT.cpp,
    tfhe_blindRotateAndExtract/mulByXaiOrCopy.cpp; stand-ins for the Xilinx
    HLS headers (ap_int.h, hls_stream.h, ap_fixed.h, ap_axi_sdata.h,
    hls_print.h) in shim_hls/; driver ref_driver_hls.cpp.
  * libref_tfhe.so -- kernel/src/{numeric-functions, lwe-functions,
    lwe-keyswitch-functions}.cpp; stand-ins for the upstream TFHE type
    headers in shim_tfhe/; driver ref_driver_tfhe.cpp.

Test infrastructure only (oracle pins).  Does nothing when the reference is
not on this machine.  The reference's testbenches, OpenCL host code and
prebuilt binaries are not used.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# the reference checkout: TFHE_REFERENCE_DIR, else the usual mount point of
# the read-only reference on the build machine
REF = os.environ.get("TFHE_REFERENCE_DIR", "/root/reference")
SRC = os.path.join(REF, "kernel", "src")

HLS_SOURCES = [os.path.join(SRC, "tfhe_blindRotate_FFT", f) for f in (
    "tGswFFTExternMulToTLwe.cpp", "pease_fft.cpp", "TorusPolynomial_fft.cpp", "tLweFromFFTConvert.cpp",
    "tfhe_MuxRotate_FFT.cpp", "tfhe_blindRotate_FFT.cpp", "tGswTorus32PolynomialDecompH.cpp",
    # linked only: the by-value tGswFFTExternMulToTLwe refers to them; both
    # carry known defects (IntPolynomial_ifft.cpp:7 writes past its output,
    # tLweFFTAddMulRTo.cpp:20 assigns where it should accumulate), and
    # nothing here calls them
    "IntPolynomial_ifft.cpp", "tLweFFTAddMulRTo.cpp")] + [
    os.path.join(SRC, "tfhe_bootstrap_woKS_FFT", "tfhe_bootstrap_woKS_FFT.cpp"),
    os.path.join(SRC, "tfhe_blindRotateAndExtract", "mulByXaiOrCopy.cpp"),
    os.path.join(HERE, "ref_driver_hls.cpp")]
TFHE_SOURCES = [os.path.join(SRC, f) for f in (
    "numeric-functions.cpp", "lwe-functions.cpp", "lwe-keyswitch-functions.cpp")] + [
    os.path.join(HERE, "ref_driver_tfhe.cpp")]

FLAGS = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-ffp-contract=off"]


def available():
    return os.path.isdir(SRC)


def _build(name, sources, includes, quiet):
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, name)
    deps = sources + [os.path.abspath(__file__)] + [
        os.path.join(d, f) for d in includes if d.startswith(HERE) for f in os.listdir(d)]
    if os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(s) for s in deps):
        return lib
    cmd = FLAGS + sum((["-I", d] for d in includes), []) + sources + ["-o", lib + ".tmp"]
    if not quiet:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build(quiet=False):
    """Build both libraries; returns their paths, or None without the reference."""
    if not available():
        return None
    hls = _build("libref_hls.so", HLS_SOURCES,
                 [os.path.join(HERE, "shim_hls"), os.path.join(SRC, "include")], quiet)
    tfhe = _build("libref_tfhe.so", TFHE_SOURCES, [os.path.join(HERE, "shim_tfhe")], quiet)
    return hls, tfhe


if __name__ == "__main__":
    print(build(quiet="--quiet" in sys.argv))
