"""Builds the reference's own CUDA kernels as GPU-side oracles (TEST INFRASTRUCTURE ONLY).

    python -m oracle.ref_build [-f]

Three reference sources are compiled UNCHANGED, from where they lie in the
reference checkout, into sm_103a cubins under ``oracle/_ref/``:

    sol_nglod.cubin     sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu
                        (aabb_kernel<float>, aabb_kernel<double>)
    spc_raytrace.cubin  sol-renderer/include/spc/spc/spc_raytrace_cuda_kernel.cu
                        (d_ScanNodesA, d_InitNuggets, d_Decide, d_Subdivide,
                        d_Compactify, d_generate_rays, and the Order table)
    sdf.cubin           sol-renderer/SDF.cu with the solr headers it includes
                        (index_trinket_kernel, sparse_grid_sample_kernel,
                        step_kernel, ray_aabb_kernel, normalize_kernel)

Only device code is compiled (``nvcc -cubin``): a cubin is GPU code and does
not depend on the host CPU, so the files built here load on the aarch64 GPU
host as they are.  The reference's host code (libtorch glue, CUB scans, GL
viewer) is not built; ``oracle/refkern.py`` restates it around these kernels.

Flags follow the reference's own builds: no fast-math and nvcc's default
floating-point contraction (``sdf-net/lib/extensions/sol_nglod/setup.py``
passes only ``-std=c++14``; ``sol-renderer/CMakeLists.txt`` adds no CUDA
flags).  C++17 is needed by today's torch headers; it does not change device
arithmetic.  The SPC sources also need ``-DCUB_NS_QUALIFIER=::kaolin::cub``
(CCCL refuses their ``CUB_NS_PREFIX`` without it) and ``oracle/ref_shim/
helper_math.h`` (the CUDA samples header they include is not installed).

``sol-renderer/sdfRenderer.cu`` (``d_MarkUniqueRays``) is not built: it
includes the GLEW and CUDA-samples GL headers, and there is no graphics stack
here.  ``refkern.mark_unique_rays`` restates that one-line kernel.

The build runs only where the reference checkout exists (this container);
elsewhere ``build()`` keeps the cubins already in ``oracle/_ref/``.  The
manifest ``oracle/_ref/manifest.json`` records each source's SHA-256, the
nvcc command and the entry functions ptxas compiled.
"""
import concurrent.futures as cf
import hashlib
import json
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
REFERENCE = os.environ.get("NGLOD_REFERENCE", "/root/reference")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
TORCH_DEFS = ["-DTORCH_API_INCLUDE_EXTENSION_H", "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
              "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__"]

# name -> (source relative to the reference root, extra defines, include dirs relative to the root)
SOURCES = {
    "sol_nglod": ("sdf-net/lib/extensions/sol_nglod/sol_nglod_kernel.cu",
                  TORCH_DEFS + ["-DTORCH_EXTENSION_NAME=sol_nglod"], []),
    "spc_raytrace": ("sol-renderer/include/spc/spc/spc_raytrace_cuda_kernel.cu",
                     ["-DCUB_NS_QUALIFIER=::kaolin::cub"], []),
    "sdf": ("sol-renderer/SDF.cu", [],
            ["sol-renderer", "sol-renderer/include/solr", "sol-renderer/third-party/cnpy"]),
}


def cubin_path(name):
    return os.path.join(OUT, name + ".cubin")


def manifest_path():
    return os.path.join(OUT, "manifest.json")


def available():
    """True when every cubin and the manifest are present."""
    return os.path.exists(manifest_path()) and all(os.path.exists(cubin_path(n)) for n in SOURCES)


def _torch_includes():
    import torch
    base = os.path.join(os.path.dirname(torch.__file__), "include")
    return [base, os.path.join(base, "torch", "csrc", "api", "include"), sysconfig.get_paths()["include"]]


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _entries(ptxas_log):
    out = []
    for line in ptxas_log.splitlines():
        key = "Compiling entry function '"
        if key in line:
            out.append(line.split(key, 1)[1].split("'", 1)[0])
    return out


def build(force=False, verbose=False):
    """Compile the cubins when the reference checkout is present; returns the
    manifest dict, or None where neither the checkout nor prebuilt cubins exist."""
    if not os.path.isdir(REFERENCE):
        if available():
            with open(manifest_path()) as f:
                return json.load(f)
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT, exist_ok=True)
    incs = _torch_includes()
    old = {}
    if os.path.exists(manifest_path()):
        with open(manifest_path()) as f:
            old = json.load(f).get("kernels", {})
    jobs = {}
    for name, (rel, defs, rinc) in SOURCES.items():
        src = os.path.join(REFERENCE, rel)
        sha = _sha(src)
        if not force and os.path.exists(cubin_path(name)) and old.get(name, {}).get("sha256") == sha:
            continue
        cmd = [nvcc, "-cubin", *ARCH, "-std=c++17", "--expt-relaxed-constexpr", "-Xptxas", "-v", *defs,
               *["-I" + p for p in incs], "-I" + SHIM, *["-I" + os.path.join(REFERENCE, p) for p in rinc],
               "-o", cubin_path(name), src]
        jobs[name] = (cmd, rel, sha)

    def run(item):
        name, (cmd, rel, sha) = item
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference kernel build failed for {rel}:\n{r.stdout}\n{r.stderr}")
        return name, {"source": rel, "sha256": sha, "command": " ".join(os.path.basename(c) if i == 0 else c
                                                                         for i, c in enumerate(cmd)),
                      "entries": _entries(r.stdout + r.stderr)}

    kernels = dict(old)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for name, rec in ex.map(run, jobs.items()):
                kernels[name] = rec
    ver = subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout.strip().splitlines()[-1]
    man = {"nvcc": ver, "arch": "sm_103a", "kernels": kernels}
    with open(manifest_path(), "w") as f:
        json.dump(man, f, indent=1)
    return man


if __name__ == "__main__":
    m = build(force="-f" in sys.argv, verbose="-v" in sys.argv)
    print(json.dumps(m, indent=1) if m else "reference checkout absent and no prebuilt cubins")
