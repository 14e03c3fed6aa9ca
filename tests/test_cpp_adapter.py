"""The C++ front end (include/medyan_mech.hpp) compiled into a host program and run.

The program is built with g++ against the in-tree library; on a machine
without a GPU it must fail loudly with MECH_ERR_NO_DEVICE (exit 3), on a GPU it
must reproduce the oracle's energies and forces and minimize to 1 pN.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from picgo_gb300 import build, jitter, make_network

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_network(net, d):
    def w(name, a, dt):
        np.ascontiguousarray(a, dtype=dt).tofile(os.path.join(d, name + ".bin"))
    w("coord", net.coord, np.float64)
    w("fil_cyl_start", net.fil_cyl_start, np.int32)
    w("cyl_bead", np.stack([net.cyl_b1, net.cyl_b2], 1), np.int32)
    w("cyl_id", net.cyl_id, np.int64)
    w("cyl_filament_id", net.cyl_fil, np.int32)
    w("cyl_position", net.cyl_pos, np.int32)
    w("cyl_type", net.cyl_type, np.int32)
    w("cyl_eq_length", net.cyl_l0, np.float64)
    w("cyl_k_stretch", net.cyl_kstr, np.float64)
    w("cyl_k_bend", net.cyl_kbend, np.float64)
    w("cyl_eq_theta", net.cyl_theta0, np.float64)
    w("cyl_k_exvol", net.cyl_kexvol, np.float64)
    w("lk_cyl", net.lk_cyl, np.int32)
    w("lk_pos", net.lk_pos, np.float64)
    w("lk_k", net.lk_k, np.float64)
    w("lk_eq_length", net.lk_l0, np.float64)
    w("planes", net.planes, np.float64)
    w("plane_k", net.plane_k, np.float64)
    w("plane_screen", net.plane_slen, np.float64)
    w("misc", [net.box, net.exvol_cutoff, net.boundary_cutoff], np.float64)


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path_factory.mktemp("cpp") / "adapter_check")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"), "-L", libdir, "-lmedyan_mech",
           "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def small_network():
    net = make_network("c1", n_filaments=24, n_cyl_per_filament=10, box=1400.0, n_linkers=40, n_motors=0)
    return jitter(net, 0.3, seed=7)


def run(program, net, tmp_path, precision=0):
    write_network(net, str(tmp_path))
    return subprocess.run([program, str(tmp_path), str(precision)], capture_output=True, text=True, timeout=600)


def test_program_builds_and_fails_loudly_without_device(program, tmp_path):
    torch = pytest.importorskip("torch")
    r = run(program, small_network(), tmp_path)
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
    else:
        assert r.returncode == 3, (r.returncode, r.stdout, r.stderr)
        assert "MECH_ERR" in r.stderr or "device" in r.stderr


@pytest.mark.gpu
def test_program_matches_oracle(program, tmp_path):
    net = small_network()
    r = run(program, net, tmp_path)
    assert r.returncode == 0, r.stderr
    rd = lambda n: np.fromfile(os.path.join(str(tmp_path), n + ".bin"), dtype=np.float64)
    per = rd("out_energies")
    vec = oracle.vectorize(net)
    with oracle.series_atan_mode():
        o_tot, o_per = oracle.energies(vec, net.coord)
        fo = oracle.forces(vec, net.coord)
        scale = oracle.force_scale(vec, net.coord)
    assert np.all(np.abs(per[:6] - o_per) <= 1e-12 * np.abs(o_per) + 1e-10), (per, o_per)
    f = rd("out_forces").reshape(-1, 3)
    assert np.all(np.abs(f - fo) <= 1e-12 * scale + 1e-9)
    status, maxf, iters, e_after = rd("out_result")
    assert status == 0 and maxf < 1.0, (status, maxf, iters)
    fmin = rd("out_min_forces").reshape(-1, 3)
    assert np.abs(fmin).max() == pytest.approx(maxf, rel=1e-12)
    xmin = rd("out_coord").reshape(-1, 3)
    assert oracle.energy(vec, xmin) == pytest.approx(e_after, rel=1e-10)
