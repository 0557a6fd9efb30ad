"""The header-only C++ layer (include/split_gb300.hpp): a program written
against the reference's names compiles and links against the library here,
and on the GPU its stage outputs equal the oracle's."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
import split_synth as synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "sample_pipeline.cpp")


def _compile(out_dir):
    from split_gb300 import build
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    lib = build.build_library()
    exe = os.path.join(str(out_dir), "sample_pipeline")
    libdir = os.path.dirname(lib)
    sdir = os.path.dirname(synth.build())
    cmd = [nvcc, "-std=c++17", "-O2", "-x", "c++", SRC, "-I", os.path.join(ROOT, "include"),
           "-L", libdir, "-lsplit_gb300", "-Xlinker", f"-rpath={libdir}",
           "-L", sdir, "-lsplit_synth", "-Xlinker", f"-rpath={sdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_layer_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


def _read(d, name, dtype, shape):
    return np.fromfile(os.path.join(d, name), dtype=dtype).reshape(shape)


@pytest.mark.gpu
def test_cpp_sample_pipeline_matches_oracle(tmp_path, cuda):
    w, h, k, iters, seed = 320, 240, 8, 10, 1234
    exe = _compile(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([exe, str(out), str(w), str(h), str(k), str(iters), str(seed)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    info = json.loads(r.stdout.strip().splitlines()[-1])
    assert info["iterations"] == iters
    n = w * h
    rgb = synth.voronoi_rgb8(seed, w, h, 32, npalette=0, illum_gradient=False, sigma=4.0)
    feats = synth.features(rgb, 3)
    c_in = _read(out, "centroids_in.f32", np.float32, (3, k))
    assert np.array_equal(c_in, synth.pick_centroids(seed, rgb, k, 3))
    km = _read(out, "kmeans_labels.i32", np.int32, (n,))
    cen = _read(out, "centroids.f32", np.float32, (3, k))
    # the returned centroids are the FP64 member means of the returned labels
    # (within 1e-5 relative), and the C++ layer equals the Python binding
    ref_c, cnt = oracle.kmeans_update_f64(km, feats, cen)
    assert (cnt > 0).all()
    assert (np.abs(cen - ref_c) / np.maximum(np.abs(ref_c), 1e-30)).max() <= 1e-5
    import torch
    from split_gb300 import kmeans
    lab = torch.empty(n, dtype=torch.int32, device=cuda)
    cd = torch.from_numpy(c_in.copy()).to(cuda)
    kmeans.cluster(torch.from_numpy(feats).to(cuda), cd, lab, None, max_iter=iters,
                   threshold=-1.0, layout=0, dim=3, width=w)
    assert np.array_equal(lab.cpu().numpy(), km)
    assert np.array_equal(cd.cpu().numpy(), cen)
    # cluster(..., 100, 1e-3) through the C++ layer uses the reference's
    # convergence rule: the same stop as the binding with that rule, and as
    # the oracle's restatement of it
    its = torch.zeros(1, dtype=torch.int32, device=cuda)
    cd2 = torch.from_numpy(c_in.copy()).to(cuda)
    kmeans.cluster(torch.from_numpy(feats).to(cuda), cd2, lab, None, max_iter=100,
                   threshold=1e-3, layout=kmeans.PLANAR | kmeans.REFERENCE_SHIFT, dim=3,
                   width=w, iterations_out=its)
    assert info["iterations_thr"] == int(its.item())
    assert oracle.kmeans_cluster_threshold(feats, c_in, 100, 1e-3)[2] == info["iterations_thr"]
    assert np.array_equal(_read(out, "kmeans_thr_labels.i32", np.int32, (n,)), lab.cpu().numpy())
    assert np.array_equal(_read(out, "centroids_thr.f32", np.float32, (3, k)), cd2.cpu().numpy())
    # every stage after k-means is bit-exact given its input
    seg = _read(out, "ccl.i32", np.int32, (h, w))
    assert np.array_equal(seg, oracle.ccl(km.reshape(h, w), 4, 1))
    comp = _read(out, "compressed.i32", np.int32, (h, w))
    ref_comp, nseg = oracle.compress_labels(seg)
    assert np.array_equal(comp, ref_comp.reshape(h, w)) and nseg == info["segments"]
    merged = _read(out, "merged.i32", np.int32, (h, w))
    assert np.array_equal(merged, oracle.merge_small(comp, 64, 1, feats[:2]))
    eroded = _read(out, "eroded.i32", np.int32, (h, w))
    assert np.array_equal(eroded, oracle.erode(merged, 1))
    nrm = _read(out, "normals.f32", np.float32, (3, n))
    ref_n = oracle.sobel_normals_f64(feats[0].reshape(h, w), 1.0)
    got = nrm.astype(np.float64)
    ref_n = ref_n.reshape(3, n)
    # angle from atan2(|a x b|, a . b): well conditioned near zero
    ang = np.arctan2(np.linalg.norm(np.cross(got.T, ref_n.T), axis=1), (got * ref_n).sum(0))
    assert ang.max() <= 1e-4
