"""Builds oracle/_ref/libref_*.so: the reference's own source for the TSDF ->
mesh path, compiled for the host CPU, to check the oracle against.  TEST
INFRASTRUCTURE ONLY.

The reference is CUDA written for a Fermi-era toolkit; its kernels cannot be
built with CUDA 13 (texture references, non-_sync warp votes) and most of
the KinectFusion part sits inside `#if 0`.  The functions on the path are,
however, plain arithmetic over arrays.  This recipe takes them out of the
reference files by line range (each range checked against a SHA-256 of its
text, so a changed reference fails loudly instead of building something
else), writes each into oracle/_ref/gen/ behind a #line directive, and
compiles two harness units that include them -- with g++, against the
reference's own headers (cu_vector_functions.h, cu_geometry_functions.h,
cu_memory.hpp, structure.h, cu_kinect_fusion_v1.h) and the CUDA toolkit's
host headers, with oracle/ref/shim/ standing in for the CUDA samples'
helper headers and for the device built-ins:

  ref_live.cpp   the live marching-cubes code: CubeIndexEstimator
                 (cu_marching_cubes_v1.cu:49-95), TrianglesGenerator
                 (:228-370), the tables (:469-1028), and the surface normals
                 (cu_kinect_fusion_v1.cu:3146-3242)
  ref_dead.cpp   the KinectFusion code inside #if 0: depth -> metre / vertex /
                 normal maps (cu_kinect_fusion_v1.cu:95-151), voxel
                 initialisation (:364-379), depth scaling and volumetric
                 integration (:416-532), the RLE slice codec (:1362-1447), with
                 the self-consistent pack / unpack pair (cu_kinect_fusion_v1.h:
                 152-171) and a 4-byte voxel (the live structure.h type; the
                 dead code's colour member is a placeholder that stores nothing)

Each unit becomes its own library (libref_live.so, libref_dead.so), built
twice: with -ffp-contract=off (every float expression as written: the
convention of the oracle and of the CUDA library) and, as libref_*_fma.so,
with -ffp-contract=fast (multiply-adds fused where the compiler may, as nvcc
does by default), for measuring how far contraction moves the reference's
own results.

    python oracle/ref/build_ref.py [REFERENCE_ROOT]      (default /root/reference)

Only oracle/_ref/ is written.  Returns without building when the reference
tree is absent (the tests that need the library skip then).
"""
import hashlib
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
GEN = os.path.join(OUT, "gen")
DEFAULT_ROOT = "/root/reference"

MC = "cu_marching_cubes_v1.cu"
KF = "cu_kinect_fusion_v1.cu"
KFH = "cu_kinect_fusion_v1.h"
ST = "structure.h"

# name, reference file, first line, last line (inclusive), sha256 of the lines
RANGES = [
    ("mc_textures", MC, 31, 33, "066ef1d1758460e11ae194cc3aaf3e4e593fff3d1ebad8223f8c67934de71935"),
    ("mc_cube_index", MC, 49, 95, "75bc7fe2749642bfaed9e935df9b35ddcdfaf8c3c92bad1f67230ad68546a516"),
    ("mc_generator", MC, 228, 370, "2ed7c996211a2b719451c49bfb2506ce93c15ff5ef24a5323869837267af11e5"),
    ("mc_tables", MC, 469, 1028, "b15df76799f70eccc58fd72f89aa61ad101ee2eedb84568267d08d9d4262f619"),
    ("kf_normals", KF, 3146, 3242, "0051ed7a46948cd9bcdae5ad51751a50df1970dc995825dbe755d4c58b6be401"),
    ("kf_depth_maps", KF, 95, 151, "ba7d1f5138127b62f97edeec963fd99e580050cbacb251696e12d2258ba49495"),
    ("kf_voxel_init", KF, 364, 379, "ec281c7d3024d2b365e79fb603f421818bd2fec3e8dfad182b7ab92ea085df7c"),
    ("kf_integrate", KF, 416, 532, "282cdd46d30abfd2b86551f376703c92640ec6899e048b94e3732e0ea55576a1"),
    ("kf_rle", KF, 1362, 1447, "de108a2b321a4dacb65c1706520401c2e0f34e25bc30254450cdc2b470540544"),
    ("kfh_consts", KFH, 30, 46, "b88aa6d6474d21120052fc201ed76aba889684123e3b2246d8a608d1a13d64d7"),
    ("kfh_pack", KFH, 152, 171, "ecd44879b8e53f59e9772e4135024500e49ca05594ee93780e77266fcfcabf73"),
    ("st_volume", ST, 20, 39, "69972f9084ad4c4cea94fb535a21b16ccb2fc27ce9a53a2f5eb83dcf737bfcd8"),
]


def extract(root, check=True):
    os.makedirs(GEN, exist_ok=True)
    digests = {}
    for name, fname, a, b, want in RANGES:
        path = os.path.join(root, fname)
        with open(path, "r", encoding="latin-1") as f:
            lines = f.readlines()
        if b > len(lines):
            raise SystemExit("%s: %s has %d lines, range ends at %d" % (name, fname, len(lines), b))
        text = "".join(lines[a - 1:b])
        d = hashlib.sha256(text.encode("latin-1")).hexdigest()
        digests[name] = d
        if check and want and d != want:
            raise SystemExit("%s: %s:%d-%d changed (sha256 %s, expected %s)" % (name, fname, a, b, d, want))
        with open(os.path.join(GEN, name + ".inc"), "w", encoding="latin-1") as f:
            f.write('#line %d "%s"\n' % (a, path))
            f.write(text)
    return digests


def compile_lib(root, fma):
    cxx = os.environ.get("CXX", "g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    flags = ["-std=c++20", "-O2", "-fPIC", "-shared", "-w", "-fno-fast-math",
             "-include", os.path.join(HERE, "shim", "ref_device.h"),
             "-I" + os.path.join(HERE, "shim"), "-I" + GEN, "-I" + root, "-I" + cuda_inc]
    if fma:
        flags.append("-ffp-contract=fast")
        if platform.machine() in ("x86_64", "AMD64"):
            flags.append("-mfma")  # aarch64 has fused multiply-add in its base ISA
    else:
        flags.append("-ffp-contract=off")
    # one library per unit: the two units see different definitions of the
    # reference's voxel and weight unpacking (live vs #if 0 code), which must
    # not meet at link time
    outs = []
    for unit in ("live", "dead"):
        out = os.path.join(OUT, "libref_%s%s.so" % (unit, "_fma" if fma else ""))
        src = os.path.join(HERE, "ref_%s.cpp" % unit)
        r = subprocess.run([cxx] + flags + [src, "-o", out + ".tmp"], capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit("reference host build failed:\n" + r.stdout + r.stderr)
        os.replace(out + ".tmp", out)
        outs.append(out)
    return outs


def build(root=None, check=True):
    root = root or os.environ.get("MCG_REFERENCE_ROOT", DEFAULT_ROOT)
    if not os.path.isfile(os.path.join(root, MC)):
        return None
    extract(root, check)
    return compile_lib(root, False) + compile_lib(root, True)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--digests":
        root = sys.argv[2] if len(sys.argv) > 2 else DEFAULT_ROOT
        for k, v in extract(root, check=False).items():
            print(k, v)
    else:
        print(build(sys.argv[1] if len(sys.argv) > 1 else None))
