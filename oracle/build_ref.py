"""Recipe: compile the reference's own CUDA kernels into cubins (checker only).

TEST INFRASTRUCTURE ONLY.  The reference rasteriser exists only as CUDA code
(submodules/gsplat/cuda/csrc/*.cu); it has no CPU blend.  To compare the GB300
kernels with the reference itself, and to time the reference's kernels on the
same GPU, this recipe compiles the device code of the reference's sources, where
they lie in a checkout of the reference, with the reference's own nvcc flags
(-O3 --use_fast_math --expt-relaxed-constexpr, submodules/setup.py:76-91) into
cubins under oracle/_ref/.  No reference source is copied; the cubins are build
outputs (git-ignored) that oracle/ref_gpu.py loads through the CUDA driver API.
The reference's host code (pybind/torch wrappers, cub sort) is not built: its
kernels are launched with the reference's own launch shapes, and its cub sort
is replaced by a stable sort, which defines the same order.

Usage:  python oracle/build_ref.py /path/to/reference
        (or set UBS_REFERENCE_ROOT to the checkout and omit the argument)
"""
import concurrent.futures as cf
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SOURCES = [
    "fully_fused_projection_fwd.cu",
    "fully_fused_projection_bwd.cu",
    "isect_tiles.cu",
    "rasterize_to_pixels_fwd.cu",
    "rasterize_to_pixels_bwd.cu",
    "cond_mean_convariance_opacity_fwd.cu",
    "cond_mean_convariance_opacity_bwd.cu",
    "rot_scale_l_triangle_to_covar_fwd.cu",
    "rot_scale_l_triangle_to_covar_bwd.cu",
    "l_triagnle_to_rotmat_fwd.cu",
    "l_triagnle_to_rotmat_bwd.cu",
]


def csrc_dir(ref_root):
    return os.path.join(ref_root, "submodules", "gsplat", "cuda", "csrc")


def reference_root(arg=None):
    """The reference checkout: the argument, else $UBS_REFERENCE_ROOT, else None."""
    return arg or os.environ.get("UBS_REFERENCE_ROOT") or None


def build(ref_root=None, force=False, verbose=False):
    """Compile the cubins from the checkout at ref_root (or $UBS_REFERENCE_ROOT);
    returns the output folder, or None when no checkout is given or found."""
    ref_root = reference_root(ref_root)
    if ref_root is None:
        return None
    csrc = csrc_dir(ref_root)
    if not os.path.isdir(csrc):
        return None
    os.makedirs(OUT, exist_ok=True)
    import torch.utils.cpp_extension as cpp
    incs = ["-I" + csrc, "-I" + os.path.join(csrc, "third_party", "glm")]
    incs += ["-I" + p for p in cpp.include_paths()]
    incs += ["-I" + sysconfig.get_paths()["include"]]
    nvcc = os.environ.get("NVCC", "nvcc")
    flags = ["-cubin", "-gencode", "arch=compute_103,code=sm_103", "-O3", "--use_fast_math",
             "--expt-relaxed-constexpr", "-std=c++17", "-diag-suppress", "20012,186,177,550",
             # defines torch's CUDAExtension adds to every nvcc call
             "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
             "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__"]
    jobs = []
    for src in SOURCES:
        path = os.path.join(csrc, src)
        out = os.path.join(OUT, src[:-3] + ".cubin")
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(path):
            continue
        jobs.append([nvcc] + flags + incs + [path, "-o", out])

    def run(cmd):
        if verbose:
            print(" ".join(cmd[-3:]), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference cubin build failed: %s\n%s" % (cmd[-3], r.stderr[-3000:]))

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    return OUT


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = reference_root(args[0] if args else None)
    if root is None:
        sys.exit("usage: build_ref.py /path/to/reference (or set UBS_REFERENCE_ROOT)")
    print(build(root, force="--force" in sys.argv, verbose=True))
