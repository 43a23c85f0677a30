"""Write the golden fixtures of tests/golden/ by running the reference's own
DiffMC / DiffDMC (its Python API over its CUDA extension) on the cases of
cases.py.  Needs a GPU and a reference checkout; the extension is built by
oracle/build_ref.py.

    python tests/golden/make_golden.py --ref-src <reference checkout> --out tests/golden/fixtures

Each fixture is an .npz with the inputs, the reference's verts and faces (face
indices stored as int32, their torch dtype in ``faces_dtype``) and, when the case
has a loss, its gradients (stored sparsely: flat indices + values of the non-zero
entries).  The loss weights are regenerated from the case seed; the fixture keeps
their sha256.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from cases import CASES, loss_weights, make_inputs  # noqa: E402


def sparse(a):
    flat = a.reshape(-1)
    nz = np.nonzero(flat)[0]
    return nz.astype(np.int64), flat[nz]


def run_case(diso, case, device="cuda"):
    import torch

    dt = getattr(torch, case["dtype"])
    sdf_np, def_np = make_inputs(case)
    sdf = torch.tensor(sdf_np, device=device, requires_grad=True)
    deform = torch.tensor(def_np, device=device, requires_grad=True) if def_np is not None else None
    if case["method"] == "mc":
        ext = diso.DiffMC(dtype=dt).to(device)
        verts, faces = ext(sdf, deform, isovalue=case["iso"], normalize=case["normalize"])
    else:
        ext = diso.DiffDMC(dtype=dt).to(device)
        verts, faces = ext(sdf, deform, isovalue=case["iso"], return_quads=case["return_quads"],
                           normalize=case["normalize"])
    out = dict(sdf=sdf_np, verts=verts.detach().cpu().numpy(), faces=faces.cpu().numpy().astype(np.int32),
               faces_dtype=str(faces.dtype), meta=json.dumps(case))
    if def_np is not None:
        out["deform"] = def_np
    if case["loss"] is not None and verts.shape[0] > 0:
        if case["loss"] == "sum":
            loss = verts.sum()
        else:
            w = loss_weights(case, verts.shape[0])
            out["weights_sha256"] = np.array(hashlib.sha256(w.tobytes()).hexdigest())
            loss = (verts * torch.tensor(w, device=device)).sum()
        loss.backward()
        out["grad_sdf_idx"], out["grad_sdf_val"] = sparse(sdf.grad.cpu().numpy())
        if deform is not None:
            out["grad_deform_idx"], out["grad_deform_val"] = sparse(deform.grad.cpu().numpy())
    torch.cuda.synchronize()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True)
    ap.add_argument("--out", default=os.path.join(HERE, "fixtures"))
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    from oracle.build_ref import load_reference

    diso = load_reference(args.ref_src)
    os.makedirs(args.out, exist_ok=True)
    for case in CASES:
        if args.only and args.only not in case["name"]:
            continue
        out = run_case(diso, case)
        np.savez_compressed(os.path.join(args.out, case["name"] + ".npz"), **out)
        print(case["name"], out["verts"].shape, out["faces"].shape, out["faces_dtype"], flush=True)


if __name__ == "__main__":
    main()
