"""The GCloudDmriSolver-compatible command line (dmri-fem-cloud_gb300/cli.py).

CPU: the argument scan follows GCloudDmriSolver.py:58-133 (flags in any order,
the reference's defaults, the reference's message on a bad value, -T2 and -q
read but not applied).  GPU: one run on a two-compartment mesh file whose
printed normalised signal matches the oracle, and the log.txt line.
"""

import importlib
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cli():
    return importlib.import_module("dmri-fem-cloud_gb300.cli")


def test_defaults_match_the_reference(cli):
    a = cli.parse_args([], out=lambda s: None)
    assert a["g"] == [0.0, 1.0, 0.0] and a["bvalue"] == 1000.0 and a["kappa"] == 1e-5
    assert (a["delta"], a["Delta"], a["k"], a["kcoeff"], a["T2"]) == (10600.0, 43100.0, 200.0, 3e-3, 1e16)
    assert a["IsDomainMultiple"] is False and a["IsDomainPeriodic"] is False and a["PeriodicDir"] == [0, 0, 0]


def test_flags_in_any_order(cli):
    lines = []
    argv = ["-gdir", "1", "0", "0", "-f", "m.msh", "-M", "1", "-b", "3000", "-d", "5000", "-D", "20000",
            "-p", "2e-5", "-k", "100", "-K", "2e-3", "-pdir", "1", "0", "1", "-T2", "50000", "-q", "1e-4",
            "-isperiodic", "0", "-N", "7"]
    a = cli.parse_args(argv, out=lines.append)
    assert a["ffile"] == "m.msh" and a["IsDomainMultiple"] is True and a["bvalue"] == 3000.0
    assert (a["delta"], a["Delta"], a["kappa"], a["k"], a["kcoeff"]) == (5000.0, 20000.0, 2e-5, 100.0, 2e-3)
    assert a["g"] == [1.0, 0.0, 0.0] and a["PeriodicDir"] == [1, 0, 1] and a["Nsteps"] == 7
    assert a["is_kcoeff_from_file"] is False and a["T2"] == 50000.0 and a["qvalue"] == 1e-4
    assert "input file: m.msh" in lines and "Something goes wrong with the inputs!" not in lines


def test_bad_value_keeps_what_was_read(cli):
    lines = []
    a = cli.parse_args(["-b", "2000", "-p", "abc", "-k", "50"], out=lines.append)
    assert lines[-1] == "Something goes wrong with the inputs!"
    assert a["bvalue"] == 2000.0 and a["kappa"] == 1e-5 and a["k"] == 200.0


def test_missing_or_hdf5_input_is_refused(cli, tmp_path):
    with pytest.raises(ValueError):
        cli.run(cli.parse_args([], out=lambda s: None), out=lambda s: None)
    with pytest.raises(ValueError, match="h5py"):
        cli.run(cli.parse_args(["-f", str(tmp_path / "mesh.h5")], out=lambda s: None), out=lambda s: None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "dmri-fem-cloud_gb300", "cli.py"), "-f", "x.h5"],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 2 and "h5py" in r.stderr


@pytest.mark.gpu
def test_cli_run_matches_oracle(pkg, lib, tmp_path):
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 8)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.5, 0.0)], [3.5])
    tags = np.where(reg == 1, 3, 2)                  # gmsh physical tags: phase = tag % 2
    mesh = tmp_path / "cyl.msh"
    pkg.meshfiles.write_msh2(mesh, xyz, tets, tags)
    argv = [sys.executable, os.path.join(ROOT, "dmri-fem-cloud_gb300", "cli.py"), "-f", str(mesh), "-M", "1",
            "-b", "2000", "-p", "3e-5", "-K", "2.5e-3", "-gdir", "0.6", "0.8", "0", "-k", "200"]
    r = subprocess.run(argv, capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    m = re.search(r"Normalized signal: ([0-9.eE+-]+)", r.stdout)
    assert m, r.stdout
    got = float(m.group(1))
    sd = oracle.duplicated_system(xyz, tets, reg, np.array([2.5e-3, 2.5e-3]), 0.0, 3e-5)
    prof = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(2000.0, prof.int4gb())
    ref = oracle.solve_duplicated(sd, prof, q, (0.6, 0.8, 0.0), 200.0)
    assert abs(got - ref.normalized) <= 6e-7 * abs(ref.normalized), (got, ref.normalized)   # 7 printed digits
    log = (tmp_path / "log.txt").read_text()
    assert "Normalized signal: %.6e" % got in log and "kappa: 3.000e-05" in log


@pytest.mark.gpu
def test_cli_strong_periodic_matches_oracle(pkg, lib, tmp_path):
    """-IsPeriodic 1 with -pdir: the strong pseudo-periodic form through the
    command line, against the oracle's folded system."""
    from oracle import strong
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 6)
    X = xyz[tets]
    c = 0.5 * (X.min(axis=1) + X.max(axis=1))
    reg = (c[:, 0] ** 2 + c[:, 1] ** 2 < 2.6 ** 2).astype(np.int32)   # cylinder on whole cubes
    tags = np.where(reg == 1, 3, 2)
    mesh = tmp_path / "box.msh"
    pkg.meshfiles.write_msh2(mesh, xyz, tets, tags)
    argv = [sys.executable, os.path.join(ROOT, "dmri-fem-cloud_gb300", "cli.py"), "-f", str(mesh), "-M", "1",
            "-IsPeriodic", "1", "-pdir", "1", "1", "1", "-b", "1500", "-p", "2e-5", "-K", "3e-3",
            "-gdir", "0.6", "0.8", "0", "-k", "200"]
    r = subprocess.run(argv, capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stderr
    m = re.search(r"Normalized signal: ([0-9.eE+-]+)", r.stdout)
    assert m, r.stdout
    got = float(m.group(1))
    prof = oracle.PGSE(10600, 43100)
    q = oracle.bvalue_to_q(1500.0, prof.int4gb())
    sd = strong.duplicated_strong(xyz, tets, reg, 3e-3, 0.0, 2e-5, [1, 1, 1], (0.6, 0.8, 0.0))
    ref = strong.solve_strong(sd, prof, q, 200.0)
    assert abs(got - ref["normalized"]) <= 6e-7 * abs(ref["normalized"]), (got, ref["normalized"])
