"""Writes tests/golden/kat.json: the known-answer values the tests pin.

* philox4x32_10: test vectors published with the Random123 library
  (Salmon et al., SC'11) for Philox4x32-10.
* notebook_run: the cosmology, geometry and values printed in the log of the
  reference's example run (example_CoLoRe.ipynb, cells 3 and 15: the model
  summary, "Particle horizon", "Present growth factor", the r range, L_box,
  dx and dk lines).  The script reads that notebook when it is available and
  keeps the values already in kat.json otherwise.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "kat.json")

PHILOX = [
    dict(ctr=["00000000"] * 4, key=["00000000"] * 2, out=["6627e8d5", "e169c58d", "bc57ac4c", "9b00dbd8"]),
    dict(ctr=["ffffffff"] * 4, key=["ffffffff"] * 2, out=["408f276d", "41c83b0e", "a20bc7c6", "6d5451fd"]),
    dict(ctr=["243f6a88", "85a308d3", "13198a2e", "03707344"], key=["a4093822", "299f31d0"],
         out=["d16cfe09", "94fdcceb", "5001e420", "24126ea1"]),
]


def from_notebook(path):
    nb = json.load(open(path))
    log = ""
    for c in nb["cells"]:
        for o in c.get("outputs", []):
            if "text" in o and "Particle horizon" in "".join(o["text"]):
                log = "".join(o["text"])
    g = lambda pat: re.search(pat, log).group(1)
    return dict(omega_M=0.3, omega_L=0.7, omega_B=0.3, h=0.7, w=-1.0, z_min=0.0001, z_max=0.15, n_grid=256,
                a_eq=g(r"a_eq=([0-9.]+)"), chi_H0=g(r"chi_H\(0\)=([0-9.E+]+)"), D_0=g(r"D_0=([0-9.]+)"),
                r_min=g(r"([0-9.]+) < r/\(Mpc/h\)"), r_max=g(r"< r/\(Mpc/h\) < ([0-9.]+)"),
                L_box=g(r"L_box = ([0-9.]+)"), dx=g(r"dx = ([0-9.E+-]+)"), dk=g(r"dk = ([0-9.E+-]+)"))


def main(nb=None):
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    data["philox4x32_10"] = PHILOX
    if nb and os.path.exists(nb):
        data["notebook_run"] = from_notebook(nb)
    json.dump(data, open(OUT, "w"), indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
