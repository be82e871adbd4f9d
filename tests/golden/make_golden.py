"""Extract the reference's own captured 3D runs into a JSON fixture.

Reads ``standard_output.txt`` and ``weak_form_output.txt`` of chandc/F90_DNS
(stdout of ``DNS_pressure_BC_3D`` on a 32x32x17 grid, Re=500, dt=0.002,
15 steps, standard vs weak-form pressure RHS) and writes the per-step
diagnostics lines (|u|max, |v|max, |w|max, E, dP/dx; 5 significant digits)
plus the run parameters printed in the header to ``reference_traces.json``.

Usage: python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import re
import sys

STEP = re.compile(r"Step\s+(\d+), t=\s*([0-9.Ee+-]+), \|u\|max=\s*([0-9.Ee+-]+), \|v\|max=\s*([0-9.Ee+-]+), "
                  r"\|w\|max=\s*([0-9.Ee+-]+), E=\s*([0-9.Ee+-]+), dP/dx=\s*([0-9.Ee+-]+)")
DIV0 = re.compile(r"Step\s+0, Max divergence:\s*([0-9.Ee+-]+)")


def parse(path):
    steps, div0 = [], None
    with open(path, encoding="utf-8", errors="replace") as f:
        for line in f:
            m = STEP.search(line)
            if m:
                steps.append(dict(step=int(m.group(1)), time=float(m.group(2)), umax=float(m.group(3)),
                                  vmax=float(m.group(4)), wmax=float(m.group(5)), energy=float(m.group(6)),
                                  dpdx=float(m.group(7))))
            m = DIV0.search(line)
            if m:
                div0 = float(m.group(1))
    return steps, div0


def main(ref):
    params = dict(nx=32, ny=32, nz=17, re=500.0, dt=0.002, xlen="2*pi", ylen="pi", u_centerline=1.5,
                  use_crank_nicolson=True, flow_control_method=1, target_pressure_gradient=0.006,
                  enable_perturbations=True, use_analytical_perturbations=True,
                  perturbation_amplitude=0.01, analytical_mode_x=1, analytical_mode_y=1, nsteps=15)
    out = {"params": params, "source": "chandc/F90_DNS standard_output.txt, weak_form_output.txt"}
    for key, fn, weak in (("standard", "standard_output.txt", False), ("weak_form", "weak_form_output.txt", True)):
        steps, div0 = parse(os.path.join(ref, fn))
        out[key] = {"use_weak_form_divergence": weak, "initial_max_divergence": div0, "steps": steps}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_traces.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(dst, len(out["standard"]["steps"]), len(out["weak_form"]["steps"]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the chandc/F90_DNS checkout>")
    main(sys.argv[1])
