"""Regenerates the golden fixtures of tests/golden/ from the REFERENCE implementation.

Builds oracle/_ref/refdriver from the reference's own core/*.cpp sources (oracle/Makefile, target `ref`;
needs the reference tree: oracle/Makefile's REF, or the OPENSPH_REFERENCE environment variable, or --ref) and
runs it in each mode below. Every fixture stores
the reference's inputs and outputs, so the tests never need the reference itself.

    python tests/golden/make_golden.py [--ref REFERENCE_TREE]
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from refbin import read_refbin  # noqa: E402

# name -> refdriver arguments (mode + mode arguments)
FIXTURES = {
    # basalt sphere: Tillotson, Continuity + Pressure + StandardAV, BH theta 0.5 octupole, PC, Courant
    "sphere_n1000": ["sphere", "1000", "1e4", "4", "1"],
    # solid impact: + SolidStress (Hooke), von Mises, Grady-Kipp damage, adaptive h
    "impact_n1200": ["impact", "1200", "5e4", "80", "5e3", "4", "5e3", "45"],
    # ideal gas sphere + Mach-3 impactor, leap-frog, no gravity
    "gas_n1500": ["gas", "1500", "80", "4"],
    # the same two runs with every time-step criterion (Courant, derivatives, acceleration, divergence)
    "impact_all_n1200": ["impact_all", "1200", "5e4", "80", "5e3", "6", "5e3", "45"],
    "gas_all_n1500": ["gas_all", "1500", "80", "6"],
    # solid impact with the AsymmetricSolver and the strain-rate correction tensor (the settings of the
    # reference's impact regression, regression/impact/impact.sph)
    "impact_asym_n1200": ["impact_asym", "1200", "5e4", "80", "5e3", "4", "5e3", "45"],
    # the basalt sphere with CachedGravity (gravity.recomputation_period 0.35 s: recomputed at t = 0 and 0.47)
    "sphere_cached_n1000": ["sphere_cached", "1000", "1e4", "6", "1", "0.35"],
    # trajectories at the benchmark's sizes (mode "<kind>_traj", last two arguments: dump interval, sample):
    # the basalt sphere of 10,000 requested particles (10,648 on the lattice), 100 steps, dumped every 10;
    # the solid impact of 200,000 + 5,000 requested particles (217,823), 10 steps, dumped after 1, 5 and 10
    "sphere_traj_n10648": ["sphere_traj", "10000", "1e4", "100", "1", "10", "1024"],
    "impact_traj_n217823": ["impact_traj", "200000", "5e4", "5000", "5e3", "10", "5e3", "45", "5", "2048"],
    # gravity only: Plummer sphere, BH theta 0.5 octupole vs brute force
    "gravity_n3000": ["gravity", "3000", "0.5", "7", "1e-3"],
    "gravity_n3000_t07": ["gravity", "3000", "0.7", "11", "1e-2"],
    # Barnes-Hut with two attractors (BarnesHut::evalAttractors): particle and attractor accelerations
    "attractors_n2000": ["attractors", "2000", "7", "1e-2"],
    # BruteForceGravity at N = 65,536 on portably generated points (accelerations of 1,024 seeded particles)
    "direct_n65536": ["direct", "65536", "17", "1e-3", "1024"],
    # symmetric finder pair set (KdTree findLowerRank + SymmetricSolver filter), variable h
    "pairs_n1500": ["pairs", "1500", "3"],
    # Tillotson EOS values on a (rho, u) grid
    "eos_tillotson": ["eos"],
    # HardSphereSolver clouds (1000 spheres of radius 400-600 m, density 2500, inflow -k r plus dispersion,
    # BH self-gravity with solid spheres, leap-frog with the acceleration criterion, max step 100 s):
    # arguments n, steps, collision handler, overlap handler, R, h, k, sigma, seed, G, max step
    "nbody_bounce_n1000": ["nbody", "1000", "10", "2", "0", "12000", "400", "1e-4", "0.05", "11", "6.67408e-11",
                           "100"],
    "nbody_merge_n1000": ["nbody", "1000", "8", "1", "1", "17000", "400", "1e-4", "0.05", "7", "6.67408e-11",
                          "100"],
    "nbody_default_n1000": ["nbody", "1000", "20", "3", "5", "14000", "400", "2e-4", "0.05", "3", "6.67408e-11",
                            "100"],
    "nbody_repel_n1000": ["nbody", "1000", "12", "3", "2", "14000", "400", "2e-4", "0.05", "3", "6.67408e-11",
                          "100"],
    "nbody_repelmerge_n1000": ["nbody", "1000", "10", "3", "3", "17000", "400", "1e-4", "0.05", "7",
                               "6.67408e-11", "100"],
    "nbody_internal_n1000": ["nbody", "1000", "12", "3", "4", "14000", "400", "2e-4", "0.05", "3",
                             "6.67408e-11", "100"],
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: oracle/Makefile's REF)")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    ref = [f"REF={args.ref}"] if args.ref else []
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"] + ref + [f"-j{os.cpu_count() or 4}"],
                   check=True)
    driver = os.path.join(REPO, "oracle", "_ref", "refdriver")
    for name, argv in FIXTURES.items():
        if args.only and name not in args.only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            out = os.path.join(tmp, "out.bin")
            subprocess.run([driver, out] + argv, check=True)
            data = read_refbin(out)
        data["driver_args"] = np.array(" ".join(argv))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, sum(v.nbytes for v in data.values()), "bytes")


if __name__ == "__main__":
    main()
