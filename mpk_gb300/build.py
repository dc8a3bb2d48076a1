"""Builds libmpk_gb300.so in-tree: host C++ with g++, kernels with nvcc for
sm_103a, translation units compiled in parallel, linked with nvcc.  The
METIS library bundled with the CUDA toolkit (libmetis_static.a) is linked
in when present (the reference's partitioner); without it the library
builds with METIS calls returning an error."""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpk_gb300.so")

HOST_SOURCES = ["graph.cc", "partition.cc", "prep.cc", "bufs.cc", "pdmpk.cc", "api.cc"]
CUDA_SOURCES = ["device.cu", "sstep.cu", "mlp.cu", "prep_gpu.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _metis_archive(nvcc):
    """The toolkit's libmetis_static.a, or None."""
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    cands = [os.path.join(root, "lib64", "libmetis_static.a")]
    tdir = os.path.join(root, "targets")
    if os.path.isdir(tdir):
        cands += [os.path.join(tdir, t, "lib", "libmetis_static.a") for t in sorted(os.listdir(tdir))]
    for c in cands:
        if os.path.exists(c):
            return c
    return None


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    metis = None if os.environ.get("MPKG_NO_METIS") else _metis_archive(nvcc)
    try:
        return _build(nvcc, metis, verbose, force)
    except RuntimeError:
        if metis is None:
            raise
        # the archive did not link (e.g. not position-independent here):
        # build without METIS
        sys.stderr.write("libmpk_gb300: linking METIS failed, building without it\n")
        return _build(nvcc, None, verbose, True)


def _build(nvcc, metis, verbose, force):
    stamp = os.path.join(BUILD, "metis.stamp")
    want = metis or "none"
    if not os.path.exists(stamp) or open(stamp).read() != want:
        force = True
        with open(stamp, "w") as f:
            f.write(want)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    inc = os.path.join(os.path.dirname(HERE), "include")
    headers += [os.path.join(inc, h) for h in os.listdir(inc) if h.endswith(".h")]
    jobs, objs = [], []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
                         *(["-DMPKG_HAVE_METIS"] if metis else []), "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for j in jobs]
    failed = False
    for j, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed = True
            sys.stderr.write("FAILED: " + " ".join(j) + "\n" + out + "\n")
        elif verbose and out:
            sys.stderr.write(out)
    if failed:
        raise RuntimeError("libmpk_gb300 build failed")
    if force or _newer(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, *([metis, "-Xlinker", "--exclude-libs,libmetis_static.a"] if metis else []), "-lcudart"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
