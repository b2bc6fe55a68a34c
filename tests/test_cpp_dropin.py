"""The C++ host drop-in (include/bns_nurates_gb300.hpp): a program written
against the reference's function names compiles, links and, on a GPU, gives
bitwise the results of the batched API."""

import os
import subprocess

import numpy as np
import pytest

import bns_nurates_gb300 as bn

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_program(tmp_path):
    libdir = os.path.join(REPO, "bns_nurates_gb300")
    exe = str(tmp_path / "dropin_point")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror",
                           "-I", os.path.join(REPO, "include"),
                           os.path.join(REPO, "tests", "cpp", "dropin_point.cpp"),
                           "-L", libdir, "-lbnsn_gb300", f"-Wl,-rpath,{libdir}", "-o", exe])
    return exe


def test_dropin_header_compiles_and_links(lib, tmp_path):
    assert os.path.exists(build_program(tmp_path))


@pytest.mark.gpu
def test_dropin_matches_batched_api(cuda, tmp_path):
    npts = 6
    exe = build_program(tmp_path)
    txt = subprocess.run([exe, str(npts)], check=True, capture_output=True, text=True).stdout
    vals = np.array([float(v) for v in txt.split()]).reshape(npts, 28 + 20 + 16)
    eos, m1 = bn.synthetic_points(20261203, npts)
    e, m = cuda.from_numpy(eos).cuda(), cuda.from_numpy(m1).cuda()
    distr = bn.distr_from_m1(m)
    pars = bn.opacity_params(True, False, True, True, True, brem_implementation=0,
                             use_NN_medium_corr=True, neglect_blocking=False)
    q = bn.gauss_legendre(10)
    grey = bn.m1_opacities(e, m, bn.opacity_flags(), pars, q, distr=distr)
    spec = bn.spectral_opacities(e, m, bn.opacity_flags(), pars, q, [10.], distr=distr,
                                 stimulated=1)
    cuda.cuda.synchronize()
    assert np.array_equal(vals[:, :28], distr.cpu().numpy().T)
    assert np.array_equal(vals[:, 28:48], grey.cpu().numpy().T)
    assert np.array_equal(vals[:, 48:], spec.cpu().numpy()[:, :, 0].T)


@pytest.mark.gpu
def test_dropin_fdi_matches_batched_api(cuda, tmp_path):
    exe = build_program(tmp_path)
    txt = subprocess.run([exe, "1", "fdi"], check=True, capture_output=True, text=True).stdout
    vals = np.array([float(v) for v in txt.split()]).reshape(7, 4)
    xs = np.array([-3.5, 0.25, 7.0, 60.0])
    for row, order in zip(vals, (-4.5, -1.5, 0, 0.5, 3, 10, 10.5)):
        assert np.array_equal(row, bn.fdi_host(order, xs)), order
