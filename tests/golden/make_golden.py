"""Writes the golden fixtures of tests/golden/.

1. trt_magic_parameter_rows.json -- the 21 (τ_s, τ_a, error_u, error_p) rows that the
   reference printed in examples/notebooks/trt_magic_parameter.ipynb (cell 2 output): D2Q9
   TRT Poiseuille, PoiseuilleFlow(ν, 1), ZeroVelocityInitialCondition, t_end = 100,
   VelocityConvergenceStoppingCriteria(1e-7).  Parsed from the notebook's JSON (read here
   from the reference checkout given on the command line); the values are the reference's
   own printed output, rounded to 6 significant digits by its DataFrame display.
2. trt_magic_parameter_table.json -- the 30 rows of the same cell's HTML table, which prints all
   seven columns of the results, including error_σ_xx (Inf in every row: the analytic σ_xx of the
   channel is zero, so its relative error divides by zero) and error_σ_xy.
3. oracle_vectors.json -- outputs of the CPU oracle on small inputs (populations after a few
   steps and error-norm rows), so that the oracle built on another machine can be checked
   against the one that was validated here.

Usage: python tests/golden/make_golden.py <reference checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def notebook_rows(ref_root):
    nb = json.load(open(os.path.join(ref_root, "examples", "notebooks", "trt_magic_parameter.ipynb")))
    rows = []
    for cell in nb["cells"]:
        for out in cell.get("outputs", []):
            text = "".join(out.get("data", {}).get("text/plain", out.get("text", "")))
            for line in text.splitlines():
                m = re.match(r"\s*│\s*(\d+)\s*│\s*([\d.e+-]+)\s*│\s*([\d.e+-]+)\s*│\s*\S+\s*│\s*([\d.e+-]+)\s*│"
                             r"\s*([\d.e+-]+)\s*│", line)
                if m:
                    rows.append({"row": int(m.group(1)), "tau_s": float(m.group(2)), "tau_a": float(m.group(3)),
                                 "error_u": float(m.group(4)), "error_p": float(m.group(5))})
        if rows:
            break
    return rows


def notebook_table(ref_root):
    """The HTML DataFrame table of the same output: <tr><th>k</th><td>τ_s</td><td>τ_a</td>
    <td>"D2Q9"</td><td>error_u</td><td>error_p</td><td>error_σ_xx</td><td>error_σ_xy</td></tr>."""
    nb = json.load(open(os.path.join(ref_root, "examples", "notebooks", "trt_magic_parameter.ipynb")))
    keys = ["tau_s", "tau_a", "quadrature", "error_u", "error_p", "error_sigma_xx", "error_sigma_xy"]
    for cell in nb["cells"]:
        for out in cell.get("outputs", []):
            html = "".join(out.get("data", {}).get("text/html", ""))
            rows = []
            for m in re.finditer(r"<tr><th>(\d+)</th>((?:<td>[^<]*</td>){7})</tr>", html):
                cells = re.findall(r"<td>([^<]*)</td>", m.group(2))
                row = {"row": int(m.group(1))}
                for k, v in zip(keys, cells):
                    row[k] = v.strip('"') if k == "quadrature" else v  # numbers kept as printed ("Inf")
                rows.append(row)
            if rows:
                return rows
    return []


def oracle_vectors():
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import oracle as O
    out = {}
    # D2Q9 TRT channel with force and walls, 3 x 8, 50 steps
    p = O.poiseuille_struct(1.0, 0.1, 0.1, 3, 8, 1.0, (1.0, 1.0), 1.0)
    cm = O.collision("TRT", [0.8, 0.5 + 0.25 / 0.3], force=True)
    bcs = [O.bc("bounce_back", "north", (1, 3), (1, 8)), O.bc("bounce_back", "south", (1, 3), (1, 8))]
    f = O.run("D2Q9", p, cm, bcs, O.initialize(O.INIT_ZERO_VELOCITY, "D2Q9", p), 0, 49,
              dt=O.problem_scalars(p)["delta_t"])
    out["d2q9_trt_poiseuille_3x8_50"] = f[:, :, 1].ravel().tolist()
    # D2Q37 MRT shear wave 6 x 6, 5 steps
    sw = O.shear_wave(6, 6, (0.6 - 0.5) / O.quadrature("D2Q37")["cs"])
    f = O.run("D2Q37", sw, O.collision("MRT", [0.6] * 4), [], O.initialize(O.INIT_EQUILIBRIUM, "D2Q37", sw), 0, 4)
    out["d2q37_mrt_shear_6x6_5"] = f[:, 2, 3].tolist()
    # D2Q9 SRT Taylor-Green vortex 16 x 16, 40 steps, error row
    tg = O.taylor_green_vortex(0.1, 1, 16, 16, static=False)
    f0 = O.initialize(O.INIT_EQ_OFFEQ, "D2Q9", tg)
    f, rows, _ = O.simulate("D2Q9", tg, O.collision("SRT", [0.8]), [], f0, 0, 40, n_steps=40)
    out["d2q9_srt_tgv_16_40_row"] = rows[-1]
    # lid-driven cavity D2Q13 SRT 7 x 6, 30 steps (all four walls, moving lid)
    ld = O.lid_driven_cavity(1.0 / 6.0, 1, 7, 6)
    lbcs = [O.bc("bounce_back", "east", (1, 7), (1, 6)), O.bc("bounce_back", "south", (1, 7), (1, 6)),
            O.bc("bounce_back", "west", (1, 7), (1, 6)), O.bc("moving_wall", "north", (1, 7), (1, 6), u=(0.005, 0.0))]
    f = O.run("D2Q13", ld, O.collision("SRT", [1.0]), lbcs, O.initialize(O.INIT_EQUILIBRIUM, "D2Q13", ld), 0, 29)
    out["d2q13_srt_cavity_7x6_30"] = f[:, 5, 0].tolist()
    return out


if __name__ == "__main__":
    ref = sys.argv[1]
    rows = notebook_rows(ref)
    assert len(rows) == 21, len(rows)
    json.dump({"source": "examples/notebooks/trt_magic_parameter.ipynb, cell 2 output", "rows": rows},
              open(os.path.join(HERE, "trt_magic_parameter_rows.json"), "w"), indent=1)
    table = notebook_table(ref)
    assert len(table) == 30, len(table)
    json.dump({"source": "examples/notebooks/trt_magic_parameter.ipynb, cell 2 output (HTML table)",
               "note": "values as printed (6 significant digits); error_sigma_xx is the string Inf",
               "rows": table}, open(os.path.join(HERE, "trt_magic_parameter_table.json"), "w"), indent=1)
    json.dump(oracle_vectors(), open(os.path.join(HERE, "oracle_vectors.json"), "w"), indent=1)
    print("wrote", len(rows), "notebook rows,", len(table), "table rows and the oracle vectors")
