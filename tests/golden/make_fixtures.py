"""Writes the golden fixtures under tests/golden/ from the reference's own
output files (run once, in a checkout that has the reference mounted):

    python tests/golden/make_fixtures.py <path of the reference checkout>

Sources (files the reference ships next to the code that produced them):
  KIcool/cooling.dat   per-step trace of KIcool/1DMHDwCC3.f90 (:249, :277)
  KIcool/bw051.dat     full 1D state written by SAVEU at nunit = 51 (:296-305)
  KIcool/time.DAT      the save times (row 51 = time of bw051.dat)
  KIcool/KIcoolbr.dat  KI equilibrium curve from KIcool/nibun.f90
  KIcool/time.DAT      also kept as text (first 60 lines): pins the D25.17
                       formatter of the output writers
  3DMHD-CfCA/INPUT3D.DAT  the shipped 3D deck: pins the deck reader
The trace is thinned (all of the first 200 steps, then every 10th) and the
state keeps every cell; values are stored exactly as parsed (float64).
"""
import os
import sys

import numpy as np

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <path of the reference checkout>")
    REF = sys.argv[1]
    ki = os.path.join(REF, "KIcool")
    trace = np.loadtxt(os.path.join(ki, "cooling.dat"))
    keep = np.r_[0:201, 201:len(trace):10, len(trace) - 1]
    keep = np.unique(keep)
    np.savez_compressed(os.path.join(OUT, "ki_cooling_trace.npz"), rows=keep, trace=trace[keep])
    bw = np.loadtxt(os.path.join(ki, "bw051.dat"))
    times = np.array([float(l.replace("D", "E")) for l in open(os.path.join(ki, "time.DAT")) if l.strip()])
    np.savez_compressed(os.path.join(OUT, "ki_bw051.npz"), state=bw, time=times[50], nsteps=5000)
    eq = np.array([[float(v) for v in l.split(",")] for l in open(os.path.join(ki, "KIcoolbr.dat")) if l.strip()])
    np.savez_compressed(os.path.join(OUT, "ki_equilibrium.npz"), n=eq[:, 0], p=eq[:, 1])
    lines = [l.rstrip("\n") for l in open(os.path.join(ki, "time.DAT"))][:60]
    with open(os.path.join(OUT, "ki_time_dat.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    deck = open(os.path.join(REF, "3DMHD-CfCA", "INPUT3D.DAT")).read()
    with open(os.path.join(OUT, "input3d_deck.txt"), "w") as f:
        f.write(deck)
    print("wrote", sorted(f for f in os.listdir(OUT) if f.endswith((".npz", ".txt"))))


if __name__ == "__main__":
    main()
