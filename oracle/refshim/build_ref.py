"""ORACLE build recipe (test infrastructure only): compiles the REFERENCE's own SuBSENSE / PAWCS / LOBSTER /
ViBe / PBAS sources into oracle/_ref/libref.so, for the CPU tests that pin the C restatement (oracle/*.c) to the
reference itself.

The reference is a CMake project that needs OpenCV; neither CMake's configure step nor OpenCV is
used here. Instead:

* the reference sources are compiled unmodified, from where they lie:
  modules/video/src/BackgroundSubtractionUtils.cpp, BackgroundSubtractorLBSP.cpp,
  BackgroundSubtractorSuBSENSE.cpp, BackgroundSubtractorPAWCS.cpp, BackgroundSubtractorLOBSTER.cpp,
  BackgroundSubtractorViBe.cpp, BackgroundSubtractorPBAS.cpp, with
  the reference's own headers (BackgroundSubtractionUtils.hpp, BackgroundSubtractorLBSP.hpp,
  BackgroundSubtractorSuBSENSE.hpp, BackgroundSubtractorPAWCS.hpp, BackgroundSubtractorLOBSTER.hpp, features2d LBSP.hpp, utils algo.hpp, math.hpp, cxx.hpp, simd.hpp,
  platform.hpp, console.hpp);
* ``litiv/utils/defines.hpp`` is the reference's ``defines.hpp.in`` with its @VARIABLES@ filled in
  (what CMake's configure_file does): no GLSL/CUDA/OpenCL, no SIMD paths (scalar code on every host),
  USE_CVCORE_WITH_UTILS on (the reference's path needs the OpenCV-based utils), POSIX aligned
  allocation;
* ``litiv/utils/opencv.hpp`` is replaced by a slim header (oracle/refshim/litiv/utils/opencv.hpp)
  that includes the reference's own sampling helpers (clampImageCoords ... getNeighborPosition_5x5,
  cut out of the reference's opencv.hpp by this script, unmodified);
* ``opencv2/*`` are project-written stand-ins (oracle/refshim/opencv2/) holding the cv types and the
  image operations the path calls, written from OpenCV's documented semantics with the same
  definitions as the C restatement (oracle/common.h);
* ``rand()`` is routed to the counter-based generator (oracle/refshim/lvshim_rand.h, force-included;
  for ViBe and PBAS also oracle/refshim/lvshim_rand_xy.h, which attributes their draws to the loop's pixel);
* oracle/refshim/ref_bridge.cpp exposes the reference classes through the same C API as the
  restatement (rsub_* / rpawcs_* / rlob_* / rvibe_* / rpbas_* beside osub_* / opawcs_* / olob_* / ovibe_* /
  opbas_*).

Run: python oracle/refshim/build_ref.py [reference root]. Outputs go to oracle/_ref/ only. The
reference root defaults to /root/reference; without it nothing is built (the GPU parity tests do not
need this library).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref.so")
DEFAULT_REF = "/root/reference"

SOURCES = ["modules/video/src/BackgroundSubtractionUtils.cpp",
           "modules/video/src/BackgroundSubtractorLBSP.cpp",
           "modules/video/src/BackgroundSubtractorSuBSENSE.cpp",
           "modules/video/src/BackgroundSubtractorPAWCS.cpp",
           "modules/video/src/BackgroundSubtractorLOBSTER.cpp"]
# compiled on its own with lvshim_rand_xy.h as well (its pixel loops name the pixel (x, y) / (x_orig, y_orig))
XY_SOURCES = ["modules/video/src/BackgroundSubtractorViBe.cpp", "modules/video/src/BackgroundSubtractorPBAS.cpp"]
INCLUDES = ["modules/video/include", "modules/features2d/include", "modules/utils/include"]
SHIM_SOURCES = ["ref_bridge.cpp", "lv_support.cpp"]

# configure values for defines.hpp.in (CMake's configure_file); anything not listed becomes 0
CONFIG = {
    "LITIV_VERSION": "0.0.0", "LITIV_VERSION_MAJOR": "0", "LITIV_VERSION_MINOR": "0", "LITIV_VERSION_PATCH": "0",
    "GIT_SHA1": "unknown", "DATASETS_CACHE_SIZE": "0", "RLUTIL_STRING_TYPE": "std::string",
    "EXTERNAL_DATA_ROOT": "/nonexistent", "SAMPLES_DATA_ROOT": "/nonexistent",
    "TEST_INPUT_DATA_ROOT": "/nonexistent", "TEST_OUTPUT_DATA_ROOT": "/nonexistent",
    "CUDA_VERSION": "0", "BUILD_SHARED_LIBS": "1", "USE_CVCORE_WITH_UTILS": "1", "USE_POSIX_ALIGNED_ALLOC": "1",
}


def configure_defines(ref, out_dir):
    src = open(os.path.join(ref, "modules/utils/include/litiv/utils/defines.hpp.in")).read()
    text = re.sub(r"@([A-Za-z0-9_]+)@", lambda m: CONFIG.get(m.group(1), "0"), src)
    dst = os.path.join(out_dir, "litiv", "utils")
    os.makedirs(dst, exist_ok=True)
    path = os.path.join(dst, "defines.hpp")
    if not os.path.exists(path) or open(path).read() != text:
        open(path, "w").write(text)


def extract_sampling_helpers(ref, out_dir):
    """The reference's clampImageCoords .. getNeighborPosition_5x5 (namespace lv of
    modules/utils/include/litiv/utils/opencv.hpp), cut at the declarations that bound them."""
    lines = open(os.path.join(ref, "modules/utils/include/litiv/utils/opencv.hpp")).read().split("\n")
    start = next(i for i, l in enumerate(lines) if "inline void clampImageCoords(" in l)
    while start > 0 and lines[start - 1].strip().startswith("///"):
        start -= 1
    end = next(i for i, l in enumerate(lines) if i > start and "void getLogPolarMask(" in l)
    while lines[end - 1].strip().startswith("///"):
        end -= 1
    block = "\n".join(lines[start:end]) + "\n"
    if "getNeighborPosition_5x5" not in block or "getSamplePosition_7x7_std2" not in block:
        raise RuntimeError("sampling helpers not found in the reference's opencv.hpp")
    path = os.path.join(out_dir, "lv_sampling_helpers.inc")
    if not os.path.exists(path) or open(path).read() != block:
        open(path, "w").write(block)


def build(ref=DEFAULT_REF, verbose=False):
    if not os.path.isdir(os.path.join(ref, "modules", "video")):
        return None
    gen = os.path.join(OUT, "gen")
    os.makedirs(gen, exist_ok=True)
    configure_defines(ref, gen)
    extract_sampling_helpers(ref, gen)
    srcs = [os.path.join(ref, s) for s in SOURCES] + [os.path.join(HERE, s) for s in SHIM_SOURCES]
    xy_srcs = [os.path.join(ref, s) for s in XY_SOURCES]
    deps = srcs + xy_srcs + [os.path.join(dp, f) for dp, _, fs in os.walk(HERE) for f in fs if f.endswith((".h", ".hpp"))]
    deps += [os.path.join(gen, "lv_sampling_helpers.inc"), os.path.join(gen, "litiv/utils/defines.hpp"),
             os.path.join(ORACLE, "philox.h"), __file__]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    # shim headers first, so that they replace opencv2/* and litiv/utils/opencv.hpp; the configured
    # defines.hpp next; then the reference's include directories
    base = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
            "-I" + HERE, "-I" + gen, "-I" + ORACLE] + ["-I" + os.path.join(ref, d) for d in INCLUDES]
    base += ["-include", os.path.join(HERE, "lvshim_rand.h")]
    objs = []
    for src in xy_srcs:
        obj = os.path.join(OUT, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = base + ["-include", os.path.join(HERE, "lvshim_rand_xy.h"), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        objs.append(obj)
    cmd = base + ["-shared", "-o", LIB] + srcs + objs + ["-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF, verbose=True))
