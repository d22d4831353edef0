"""Regenerate tests/golden/diffops_ah_n32.json and diffops_c_n32.json from
the reference's own known-answer file
src/test/test_diff_ops/reference_results.txt.

Run once in a container that has the reference checked out:
    python tests/golden/make_golden.py REFERENCE_CHECKOUT
The JSON keeps only the entries that pin the hot path -- the Ah-grid SBP
operators and the colocated pointwise operators (co2contra, contra2co,
Coriolis, kinetic energy; the last two are tested on the A grid) -- each
with the line number of the reference file it came from.  The C-grid file
keeps the SBP operators of the &shallow_water_model_c family (div, grad,
curl, Coriolis, KE and co2contra at sbp21 and sbp42) and the co2contra /
contra2co pair of co2contra_c_sbp*_new that the C-grid hyperdiffusion's curl
part uses, and gradient_a2_ecs and divergence_a2_ecs, whose halos are the
interpolating ECS_O and ecs_A_vec halos of the cell centres.  The
values were printed by the reference test with format "(A,4E15.7)", i.e. to
7 significant digits, from test_diffops_all.f90 at N=32, nz=3.
"""
import json
import os
import sys

KEEP = {
    "divergence_ah42_sbp": ("div", 42),
    "divergence_ah43_sbp": ("div", 43),
    "gradient_ah21_sbp_ecs": ("grad", 21),
    "gradient_ah42_sbp_ecs": ("grad", 42),
    "gradient_ah43_sbp_ecs": ("grad", 43),
    "curl_divergence_ah42_sbp": ("curl", 42),
    "curl_divergence_ah43_sbp": ("curl", 43),
    "co2contra_colocated Ah grid": ("co2contra", 42),
    "contra2co_colocated": ("contra2co", 42),
    "coriolis_colocated": ("coriolis", 42),
    "KE_colocated": ("ke", 42),
}

KEEP_C = {
    "divergence_c_sbp21": ("div", 21), "divergence_c_sbp42": ("div", 42),
    "gradient_c_sbp21": ("grad", 21), "gradient_c_sbp42": ("grad", 42),
    "curl_c_sbp21": ("curl", 21), "curl_c_sbp42": ("curl", 42),
    "coriolis_Cgrid_sbp21": ("coriolis", 21), "coriolis_Cgrid_sbp42": ("coriolis", 42),
    "KE_Cgrid_sbp21": ("ke", 21), "KE_Cgrid_sbp42": ("ke", 42),
    "co2contra_c_sbp21": ("co2contra", 21), "co2contra_c_sbp42": ("co2contra", 42),
    "co2contra_c_sbp21_new": ("co2contra", 21), "co2contra_c_sbp42_new": ("co2contra", 42),
    "contra2co_c_sbp21_new": ("contra2co", 21), "contra2co_c_sbp42_new": ("contra2co", 42),
    # the A grid's central-difference gradient on the cell centres, which pins
    # the ECS_O halo (the sbp_order entry only selects the oracle domain)
    "gradient_a2_ecs": ("grad_a2_ecs", 42),
    # the A grid's divergence, which pins the ecs_A_vec halo
    "divergence_a2_ecs": ("div_a2_ecs", 42),
    # the C grid's second-order gradient, with the ECS_O halo
    "gradient_c2_ecs": ("grad_c2_ecs", 42),
}


def extract(lines, keep):
    out = []
    for k, line in enumerate(lines):
        name = line.strip()
        if name in keep and k + 1 < len(lines) and lines[k + 1].startswith("Err:"):
            vals = [float(x) for x in lines[k + 1].split()[1:]]
            kind, order = keep[name]
            out.append({"name": name, "kind": kind, "sbp_order": order, "N": 32,
                        "nz": 3, "values": vals,
                        "source": f"src/test/test_diff_ops/reference_results.txt:{k + 1}-{k + 2}"})
    return out


def main(ref_root):
    path = os.path.join(ref_root, "src/test/test_diff_ops/reference_results.txt")
    lines = open(path).read().splitlines()
    here = os.path.dirname(os.path.abspath(__file__))
    for keep, fname in ((KEEP, "diffops_ah_n32.json"), (KEEP_C, "diffops_c_n32.json")):
        out = extract(lines, keep)
        dst = os.path.join(here, fname)
        with open(dst, "w") as f:
            json.dump(out, f, indent=1)
        print(f"wrote {len(out)} entries to {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
