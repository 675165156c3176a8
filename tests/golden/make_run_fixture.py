"""Write tests/golden/run_acis_i/: a small run of mx_run_marx (needs a GPU).

    python tests/golden/make_run_fixture.py [OUT_DIR]

A POINT source 30" off the aim point, FLAT 0.3-8 keV, INTERNAL dither,
ACIS-I, 20000 photons in batches of 5000, RandomSeed 7: the column files,
marx.par and obs.par of the run, which the reference's marx2fits reads in
tests/test_run.py."""
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from marx_gb300 import config as cfgmod  # noqa: E402
from marx_gb300.run import write_par, run_marx  # noqa: E402


def main(out):
    c = cfgmod.default_config()
    c.grating = cfgmod.GRATING["NONE"]
    c.detector = cfgmod.DETECTOR["ACIS-I"]
    c.dither = cfgmod.DITHER["INTERNAL"]
    with tempfile.TemporaryDirectory() as tmp:
        par = os.path.join(tmp, "sim.par")
        run_dir = os.path.join(tmp, "run")
        write_par(par, c, NumRays=20000, dNumRays=5000, OutputDir=run_dir, RandomSeed=7,
                  SourceRA=250.2134679741175 + 30.0 / 3600.0, SourceDEC=-53.75743813458669, MinEnergy=0.3,
                  MaxEnergy=8.0, SourceFlux=0.01)
        st = run_marx(par)
        if os.path.exists(out):
            shutil.rmtree(out)
        shutil.copytree(run_dir, out)
    print(out, st)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "run_acis_i"))
