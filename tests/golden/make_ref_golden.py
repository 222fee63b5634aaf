"""Generate the reference fixtures tests/golden/ref_<scenario>.npz.

Builds the reference's own sources against the project-written stand-ins of
their absent third-party libraries (oracle/refpin/build.py; it reads the
reference checkout in place and needs it present, so this script runs where
the checkout is, not on a machine without it), runs every scenario of
tests/ref_scenarios.py as a reference input script, and stores its inputs
and final state:

  atoms (tags, mol, types, x), script text;
  phi, chempot, gradx/grady/gradz ([z][y][x]);
  owned-bead x, ux, F and image flags; counters (owned beads, timestep,
  neighbor builds, Flory-Huggins reflections phi <= 0 and phi >= 1);
  the half bead list as (tag, tag, image code) rows and the grid list as
  (node, tag, image code) rows; compute arrays.

  python tests/golden/make_ref_golden.py [scenario ...]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refpin import build as RB  # noqa: E402
from tests import ref_scenarios as RS  # noqa: E402


def read_state(path):
    out = {}
    b = open(path, "rb").read()
    o = 0
    while o < len(b):
        name = b[o:o + 32].split(b"\0")[0].decode()
        o += 32
        dt, nd = np.frombuffer(b, np.int32, 2, o)
        o += 8
        dims = np.frombuffer(b, np.int64, nd, o)
        o += 8 * nd
        typ = [np.float64, np.int32, np.int64][dt]
        cnt = int(np.prod(dims)) if nd else 0
        out[name] = np.frombuffer(b, typ, cnt, o).reshape(dims).copy()
        o += cnt * np.dtype(typ).itemsize
    return out


def lists(state, sc):
    """The half bead list and the grid list as canonical rows."""
    n = int(state["counters"][0])
    x_all, tags_all = state["x"], state["tags"]
    out = {}
    k = 0
    while "list%d_ilist" % k in state:
        il, nn, nb = state["list%d_ilist" % k], state["list%d_numneigh" % k], state["list%d_neigh" % k]
        ltype = state["list%d_kind" % k][0]  # NeighList::FULL (1): grid list; HALF (0): bead pairs
        rows = []
        m = 0
        for ii, i in enumerate(il):
            js = nb[m:m + nn[ii]]
            m += nn[ii]
            if len(js) == 0:
                continue
            codes = RS.shift_codes(x_all, tags_all, n, sc["period"], js)
            for j, c in zip(js, codes):
                first = int(i) if ltype == 1 else int(tags_all[i])  # the full (grid) list holds node indices
                rows.append((first, int(tags_all[j]), int(c)))
        out["grid_list" if ltype == 1 else "half_list"] = np.asarray(rows, np.int32).reshape(-1, 3)
        k += 1
    return out


def run(name, exe):
    sc = RS.SCENARIOS[name]
    beads = RS.bead_inputs(sc)
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "atoms.data"), "w") as f:
            f.write(RS.atoms_file_text(beads))
        os.makedirs(os.path.join(tmp, "dumps"))
        text = RS.script(sc, "atoms.data", "dumps")
        with open(os.path.join(tmp, "run.in"), "w") as f:
            f.write(text)
        env = dict(os.environ, REFPIN_OUT=os.path.join(tmp, "state.bin"))
        r = subprocess.run([exe, "-in", "run.in"], cwd=tmp, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference run of %s failed: %s%s" % (name, r.stdout[-2000:], r.stderr[-2000:]))
        st = read_state(os.path.join(tmp, "state.bin"))
    n = int(st["counters"][0])
    tags, mol, types, x = beads
    fix = dict(script=np.array(text), in_tags=tags, in_mol=mol, in_types=types, in_x=x,
               phi=st["phi"], chempot=st["chempot"], gradx=st["gradx"], grady=st["grady"], gradz=st["gradz"],
               counters=st["counters"])
    if n:
        fix.update(x=st["x"][:n], ux=st["ux"][:n], f=st["f"][:n], images=st["images"])
        fix.update(lists(st, sc))
    for k, v in st.items():
        if k.startswith("compute_"):
            fix[k] = v
    path = os.path.join(HERE, "ref_%s.npz" % name)
    np.savez_compressed(path, **fix)
    return path


def main(names):
    exe = RB.build()
    if exe is None:
        raise SystemExit("the reference's sources are not available here")
    for name in names or sorted(RS.SCENARIOS):
        print(run(name, exe))


if __name__ == "__main__":
    main(sys.argv[1:])
