"""Extract the reference's printed known answers into ``tutorial_values.json``.

The reference (somax) stores no golden arrays for the QG path; the only exact numbers are
the text outputs its tutorial notebooks print.  This script reads those outputs (never the
code cells' logic) from a somax checkout and writes them, with their cell citations, as a
small JSON fixture that the tests compare the oracle against.

Usage: python tests/golden/make_tutorial_values.py <path of a somax checkout>
"""

from __future__ import annotations

import json
import pathlib
import re
import sys


def cell_text(nb_path: pathlib.Path, cell: int) -> str:
    nb = json.loads(nb_path.read_text())
    c = nb["cells"][cell]
    return "".join("".join(o.get("text", "")) for o in c.get("outputs", []))


def main(ref: str) -> None:
    ref = pathlib.Path(ref)
    tut = ref / "content" / "tutorials"
    out: dict = {}

    s = cell_text(tut / "step10_poisson_2d.ipynb", 4)
    out["poisson_dirichlet_64_l2"] = {
        "value": float(re.search(r"L2 error = ([0-9.eE+-]+)", s).group(1)),
        "source": "content/tutorials/step10_poisson_2d.ipynb cell 4",
    }
    s = cell_text(tut / "step10_poisson_2d.ipynb", 12)
    rows = re.findall(r"n=\s*(\d+)\s+Dir=([0-9.eE+-]+)", s)
    out["poisson_dirichlet_convergence"] = {
        "n": [int(n) for n, _ in rows],
        "l2": [float(v) for _, v in rows],
        "source": "content/tutorials/step10_poisson_2d.ipynb cell 12",
    }
    s = cell_text(tut / "step11_helmholtz_2d.ipynb", 6)
    rows = re.findall(r"lambda =\s*([0-9.]+)\s+max\|phi\| = ([0-9.]+)", s)
    out["helmholtz_max_abs"] = {
        "lambda": [float(l) for l, _ in rows],
        "max_abs_phi": [float(v) for _, v in rows],
        "source": "content/tutorials/step11_helmholtz_2d.ipynb cell 6",
    }
    s = cell_text(tut / "step11_helmholtz_2d.ipynb", 12)
    out["helmholtz_lambda0_vs_poisson"] = {
        "max_abs_diff": float(re.search(r":\s*([0-9.eE+-]+)", s).group(1)),
        "source": "content/tutorials/step11_helmholtz_2d.ipynb cell 12",
    }
    s = cell_text(tut / "step07_diffusion_2d.ipynb", 14)
    out["diffusion_max_abs_error"] = {
        "value": float(re.search(r"error: ([0-9.]+)", s).group(1)),
        "source": "content/tutorials/step07_diffusion_2d.ipynb cell 14",
    }
    s = cell_text(tut / "step07_diffusion_2d.ipynb", 16)
    m = re.search(r"initial = ([0-9.]+), final = ([0-9.]+)", s)
    r = re.search(r"Ratio: ([0-9.]+)", s)
    out["diffusion_energy"] = {
        "initial": float(m.group(1)),
        "final": float(m.group(2)),
        "ratio": float(r.group(1)),
        "source": "content/tutorials/step07_diffusion_2d.ipynb cell 16",
    }
    s = cell_text(tut / "step07_diffusion_2d.ipynb", 18)
    out["diffusion_dL_dnu"] = {
        "value": float(re.search(r"dL/d\(nu\) = ([0-9.eE+-]+)", s).group(1)),
        "source": "content/tutorials/step07_diffusion_2d.ipynb cell 18",
    }
    dst = pathlib.Path(__file__).with_name("tutorial_values.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_tutorial_values.py <path of a somax checkout>")
    main(sys.argv[1])
