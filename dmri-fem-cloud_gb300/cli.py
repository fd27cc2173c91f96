"""Command line compatible with the reference's ``GCloudDmriSolver.py``.

    python dmri-fem-cloud_gb300/cli.py -f mesh.msh -M 1 -b 1000 -d 10600 -D 43100 \
        -p 1e-5 -k 200 -K 3e-3 -gdir 0 1 0

Flags and defaults follow ``GCloudDmriSolver.py:52-133``: ``-f`` mesh file,
``-M`` IsDomainMultiple, ``-IsPeriodic``/``-isperiodic``, ``-N`` (read and
unused, as there), ``-b`` b-value, ``-q`` q-value (read and unused, as there:
the b-value defines the run), ``-p`` permeability, ``-D`` Delta, ``-d`` delta,
``-K`` diffusion coefficient, ``-k`` time step, ``-T2`` (read and not applied:
the reference reads it into a local and keeps ``mri_para.T2 = 1e16``,
``GCloudDmriSolver.py:115-119``, ``DmriFemLib.py:807``), ``-gdir g0 g1 g2``,
``-pdir p0 p1 p2``.  Like the reference, flags come in any order, a value that
does not parse prints ``Something goes wrong with the inputs!`` and the run
continues with the values read so far.  The run is the reference's: PGSE
f(t) (``GCloudDmriSolver.py:186-193``), ``MRI_simulation.solve`` and
``PostProcessing``, which prints the result line and appends it to ``log.txt``.

Differences: the mesh file is a gmsh ``.msh`` (2.2 / 4.1 ASCII) or DOLFIN
``.xml`` (optionally ``.zip``), whose cell markers give the compartments
(phase = marker % 2) when ``-M 1``; the reference's HDF5 input
(``GCloudDmriSolver.py:146-177``) needs h5py, which this engine does not use,
so ``.h5`` is refused with a message.  Without a diffusion tensor in the file
the diffusion coefficient is ``-K`` (default 3e-3).  The engine solves each step
with COCG to ``-rtol`` (default 1e-12, tighter than the reference's BiCGSTAB
1e-9 / 1e-10, ``GCloudDmriSolver.py:219-222``); ``-precision mixed`` selects the
mixed-precision path.  Both are additions.
"""

import importlib
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.basename(_HERE)

DEFAULTS = {
    "g": [0.0, 1.0, 0.0], "kcoeff": 3e-3, "Nsteps": 100, "bvalue": 1000.0, "kappa": 1e-5,
    "delta": 10600.0, "Delta": 43100.0, "T2": 1e16, "k": 200.0, "IsDomainPeriodic": False,
    "IsDomainMultiple": False, "PeriodicDir": [0, 0, 0], "ffile": None, "qvalue": None,
    "is_kcoeff_from_file": True, "is_T2_from_file": True, "rtol": 1e-12, "precision": "fp64",
}


def _pkg():
    root = os.path.dirname(_HERE)
    if root not in sys.path:
        sys.path.insert(0, root)
    return importlib.import_module(_PKG)


def parse_args(argv, out=print):
    """The reference's argument scan (``GCloudDmriSolver.py:58-133``): every
    flag is looked up wherever it appears; a bad value ends the scan with the
    reference's message, keeping what was read before it."""
    a = {k: (list(v) if isinstance(v, list) else v) for k, v in DEFAULTS.items()}
    try:
        for i, arg in enumerate(argv):
            if arg == "-f":
                a["ffile"] = argv[i + 1]
                out("input file: %s" % a["ffile"])
            if arg == "-M":
                a["IsDomainMultiple"] = bool(int(argv[i + 1]))
                out("IsDomainMultiple: %d" % a["IsDomainMultiple"])
            if arg in ("-IsPeriodic", "-isperiodic"):
                a["IsDomainPeriodic"] = bool(int(argv[i + 1]))
                out("IsDomainPeriodic: %d" % a["IsDomainPeriodic"])
            if arg == "-N":
                a["Nsteps"] = int(argv[i + 1])
                out("Nsteps: %d" % a["Nsteps"])
            if arg == "-b":
                a["bvalue"] = float(argv[i + 1])
                out("bvalue: %g" % a["bvalue"])
            if arg == "-q":
                a["qvalue"] = float(argv[i + 1])
                out("qvalue: %g" % a["qvalue"])
            if arg == "-p":
                a["kappa"] = float(argv[i + 1])
                out("permeability: %g" % a["kappa"])
            if arg == "-D":
                a["Delta"] = float(argv[i + 1])
                out("Delta: %g" % a["Delta"])
            if arg == "-d":
                a["delta"] = float(argv[i + 1])
                out("delta: %g" % a["delta"])
            if arg == "-K":
                a["is_kcoeff_from_file"] = False
                a["kcoeff"] = float(argv[i + 1])
                out("diffusion coefficient: %g" % a["kcoeff"])
            if arg == "-k":
                a["k"] = float(argv[i + 1])
                out("time step size: %g" % a["k"])
            if arg == "-T2":
                a["is_T2_from_file"] = False
                a["T2"] = float(argv[i + 1])
                out("T2: %g" % a["T2"])
            if arg == "-gdir":
                a["g"] = [float(argv[i + 1]), float(argv[i + 2]), float(argv[i + 3])]
                out("(g0, g1, g2): %g %g %g" % tuple(a["g"]))
            if arg == "-pdir":
                a["PeriodicDir"] = [int(argv[i + 1]), int(argv[i + 2]), int(argv[i + 3])]
                out("PeriodicDir=[ %d %d %d ]" % tuple(a["PeriodicDir"]))
            if arg == "-rtol":
                a["rtol"] = float(argv[i + 1])
            if arg == "-precision":
                a["precision"] = argv[i + 1]
                if a["precision"] not in ("fp64", "mixed"):
                    raise ValueError(a["precision"])
    except (IndexError, ValueError):
        out("Something goes wrong with the inputs!")
    return a


def run(a, out=print, logfile="log.txt", device=0):
    """The reference's run (``GCloudDmriSolver.py:146-236``) on the engine.
    Returns (PostProcessing text, MRI_simulation)."""
    pkg = _pkg()
    ffile = a["ffile"]
    if not ffile:
        raise ValueError("no input mesh: give -f <mesh.msh|mesh.xml>")
    stem = ffile[:-4] if ffile.endswith(".zip") else ffile
    if stem.endswith(".h5"):
        raise ValueError("HDF5 mesh input needs h5py, which this engine does not use: convert %s to gmsh .msh or "
                         "DOLFIN .xml" % ffile)
    mymesh = pkg.Mesh.read(ffile, compact_markers=True)
    mri_simu = pkg.MRI_simulation()
    mri_para = pkg.MRI_parameters()
    mri_para.bvalue = a["bvalue"]
    mri_para.delta, mri_para.Delta = a["delta"], a["Delta"]
    mri_para.set_gradient_dir(mymesh, *a["g"])
    mri_para.T = mri_para.Delta + mri_para.delta
    mri_para.profile = pkg.sequences.pgse(mri_para.delta, mri_para.Delta)
    mri_para.Apply()
    mri_simu.k = a["k"]
    mri_simu.nskip = 5
    mydomain = pkg.MyDomain(mymesh, mri_para)
    mydomain.PeriodicDir = list(a["PeriodicDir"])
    mydomain.IsDomainPeriodic = a["IsDomainPeriodic"]
    mydomain.IsDomainMultiple = a["IsDomainMultiple"]
    if mydomain.IsDomainMultiple and mymesh.markers is None:
        raise ValueError("-M 1 needs cell markers in the mesh file (the compartments)")
    mydomain.kappa = a["kappa"]
    mydomain.device = device
    mydomain.Apply()
    if a["is_kcoeff_from_file"]:
        out("No diffusion tensor in %s: diffusion coefficient D0 = %g" % (ffile, a["kcoeff"]))
    else:
        out("Impose diffusion coefficient from command line, D0= %g" % a["kcoeff"])
    mydomain.D0 = a["kcoeff"]
    mydomain.D = mydomain.D0
    linsolver = pkg.KrylovSolver("cocg", "jacobi")
    linsolver.parameters["relative_tolerance"] = a["rtol"]
    linsolver.parameters["maximum_iterations"] = 100000
    linsolver.parameters["precision"] = a["precision"]
    mri_simu.solve(mydomain, mri_para, linsolver)
    text = pkg.PostProcessing(mydomain, mri_para, mri_simu, None, "", logfile=logfile)
    return text, mri_simu


def main(argv=None):
    argv = sys.argv[1:] if argv is None else list(argv)
    a = parse_args(argv)
    try:
        run(a)
    except ValueError as e:
        print("error: %s" % e, file=sys.stderr)
        return 2
    return 0


if __name__ == "__main__":
    sys.exit(main())
