"""Writes tests/golden/le10_c3d20.json and le10_c3d20_fine.json.

The reference pins its stress recovery on the NAFEMS LE10 thick-plate decks
it ships as test fixtures (examples/nafems/le10_c3d20.inp and
le10_c3d20_fine.inp, generated by solver/scripts/gen_nafems.py; test
solver/src/nafems.rs:49-88).  This script reads those two decks and stores
the arrays the C ABI takes -- node coordinates, C3D20 connectivity (0-based),
material, single-point constraints as full-DOF indices, the face-pressure list
and the index of node set D -- so the tests run without the reference tree.

It understands exactly the keywords these decks use (*NODE, *ELEMENT
TYPE=C3D20, *ELSET, *NSET, *ELASTIC, *BOUNDARY, *DLOAD Pn).

Run from the repository root with the reference checked out at REF:
    python tests/golden/make_le10.py /path/to/axia-fem
"""
import json
import os
import sys


def parse(path):
    nodes, elems, sets, bcs, dloads = {}, [], {}, [], []
    e = nu = None
    mode, name, cont = None, None, []
    for raw in open(path):
        line = raw.strip()
        if not line or line.startswith("**"):
            continue
        if line.startswith("*"):
            kw = [t.strip() for t in line[1:].split(",")]
            key = kw[0].upper()
            opts = {k.split("=")[0].strip().upper(): (k.split("=")[1].strip() if "=" in k else "") for k in kw[1:]}
            mode = key
            if key == "ELEMENT":
                assert opts.get("TYPE", "").upper() == "C3D20", opts
            if key in ("NSET", "ELSET"):
                name = opts[key]
                sets[(key, name)] = []
            continue
        vals = [v.strip() for v in line.split(",") if v.strip()]
        if mode == "NODE":
            nodes[int(vals[0])] = [float(v) for v in vals[1:4]]
        elif mode == "ELEMENT":
            cont += [int(v) for v in vals]
            if len(cont) >= 21:
                elems.append(cont[:21])
                cont = cont[21:]
        elif mode in ("NSET", "ELSET"):
            sets[(mode, name)] += [int(v) for v in vals]
        elif mode == "ELASTIC":
            e, nu = float(vals[0]), float(vals[1])
        elif mode == "BOUNDARY":
            bcs.append((vals[0], int(vals[1]), int(vals[2]), float(vals[3]) if len(vals) > 3 else 0.0))
        elif mode == "DLOAD":
            dloads.append((vals[0], vals[1].upper(), float(vals[2])))
    ids = sorted(nodes)
    index = {nid: k for k, nid in enumerate(ids)}
    eids = [el[0] for el in elems]
    eindex = {eid: k for k, eid in enumerate(eids)}
    bc_dof, bc_val = [], []
    for target, d0, d1, v in bcs:
        targets = sets[("NSET", target)] if ("NSET", target) in sets else [int(target)]
        for nid in targets:
            for d in range(d0, d1 + 1):
                bc_dof.append(3 * index[nid] + d - 1)
                bc_val.append(v)
    dl_elem, dl_face, dl_p = [], [], []
    for target, face, p in dloads:
        targets = sets[("ELSET", target)] if ("ELSET", target) in sets else [int(target)]
        assert face.startswith("P")
        for eid in targets:
            dl_elem.append(eindex[eid])
            dl_face.append(int(face[1:]))
            dl_p.append(p)
    return {
        "coords": [nodes[i] for i in ids],
        "conn": [[index[n] for n in el[1:]] for el in elems],
        "e": e, "nu": nu,
        "bc_dof": bc_dof, "bc_val": bc_val,
        "dload_elem": dl_elem, "dload_face": dl_face, "dload_p": dl_p,
        "node_d": index[sets[("NSET", "D")][0]],
    }


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AXIA_REFERENCE", "")
    here = os.path.dirname(os.path.abspath(__file__))
    for deck, out in (("le10_c3d20.inp", "le10_c3d20.json"), ("le10_c3d20_fine.inp", "le10_c3d20_fine.json")):
        src = os.path.join(ref, "examples", "nafems", deck)
        d = parse(src)
        d["source"] = f"examples/nafems/{deck} (reference test fixture, solver/src/nafems.rs:49-88)"
        with open(os.path.join(here, out), "w") as fh:
            json.dump(d, fh, separators=(",", ":"))
        print("wrote", out, len(d["coords"]), "nodes", len(d["conn"]), "elements")


if __name__ == "__main__":
    main()
