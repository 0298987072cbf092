"""On-disk formats of the reference used for end-to-end parity.

* `read_vtk_polydata`: legacy VTK polydata or unstructured grid (ASCII), the mesh format of the
  reference's data sets (read by DeformableObjectReader.cxx through VTK): POINTS and POLYGONS /
  LINES / VERTICES / CELLS sections; `read_vtk_point_weights`: the one-component point-data scalars
  a point cloud takes its weights from (PointCloud.cxx:204-225).
* `read_deformation_state`: the optimiser state the reference serialises at the end of an
  estimation (FastGradientAscent.cxx:296-305 and 313-322, written by DeformationState,
  SerializeDeformationState.h) as a Boost text archive. DeformationState keeps one queue per value
  type and writes the queues in a fixed type order, so values come out grouped by type (unsigned
  ints, doubles, vectors, the named fixed-effect maps, ...) rather than in the order they were
  pushed. Matrices and vectors are written as their sizes followed by their raw doubles in
  base64 (ArmadilloMatrixWrapper.h:349-370, ArmadilloVectorWrapper.h:315-330); matrices are
  column-major.
"""
from __future__ import annotations

import base64
import re

import numpy as np

_B64 = re.compile(r"[A-Za-z0-9+/]+=*")


def read_vtk_polydata(path: str):
    """Points (n x 3 float64) and cells (list of index tuples, or an int32 array when every cell has
    the same size) of an ASCII legacy VTK polydata or unstructured-grid file (tetrahedra of
    OrientedVolumeMesh come as an unstructured grid's CELLS). Points declared `float` are rounded
    to single precision, as VTK stores them before the reference converts them to double."""
    with open(path) as f:
        tokens = f.read().split()
    i = 0
    pts = None
    cells = []
    while i < len(tokens):
        t = tokens[i].upper()
        if t == "POINTS":
            n = int(tokens[i + 1])
            vals = np.array(tokens[i + 3:i + 3 + 3 * n], dtype=np.float64)
            if tokens[i + 2].lower() == "float":
                vals = vals.astype(np.float32).astype(np.float64)
            pts = vals.reshape(n, 3)
            i += 3 + 3 * n
        elif t in ("POLYGONS", "LINES", "VERTICES", "CELLS", "TRIANGLE_STRIPS"):
            if t == "TRIANGLE_STRIPS":
                raise ValueError("triangle strips are not supported")
            m = int(tokens[i + 1])
            j = i + 3
            for _ in range(m):
                k = int(tokens[j])
                cells.append(tuple(int(v) for v in tokens[j + 1:j + 1 + k]))
                j += 1 + k
            i = j
        elif t == "BINARY":
            raise ValueError("binary VTK files are not supported")
        elif t in ("CELL_TYPES", "POINT_DATA", "CELL_DATA"):
            i += 2 + (int(tokens[i + 1]) if t == "CELL_TYPES" else 0)
            if t != "CELL_TYPES":
                break  # attribute data follows the geometry
        else:
            i += 1
    if pts is None:
        raise ValueError(f"no POINTS section in {path}")
    if cells and all(len(c) == len(cells[0]) for c in cells):
        return pts, np.array(cells, dtype=np.int32)
    return pts, cells


def read_vtk_point_weights(path: str):
    """The point-data SCALARS of a legacy VTK file as float64 (one component), or None when the
    file has none or they do not match the point count (the reference then uses unit weights,
    PointCloud.cxx:204-225)."""
    with open(path) as f:
        tokens = f.read().split()
    n_pts = None
    i = 0
    while i < len(tokens):
        t = tokens[i].upper()
        if t == "POINTS":
            n_pts = int(tokens[i + 1])
            i += 3
        elif t == "POINT_DATA":
            n = int(tokens[i + 1])
            j = i + 2
            while j < len(tokens) and tokens[j].upper() not in ("SCALARS", "CELL_DATA"):
                j += 1
            if j >= len(tokens) or tokens[j].upper() != "SCALARS":
                return None
            ncomp = 1
            j += 3  # SCALARS name type
            if j < len(tokens) and tokens[j].isdigit():
                ncomp = int(tokens[j])
                j += 1
            if j < len(tokens) and tokens[j].upper() == "LOOKUP_TABLE":
                j += 2
            if ncomp != 1 or n != n_pts:
                return None
            return np.array(tokens[j:j + n], dtype=np.float64)
        else:
            i += 1
    return None


def reorient_like_reader(pts, tris, flip: bool = True):
    """Triangle orientation the reference gives an OrientedSurfaceMesh read with re-orientation on
    (the default, DeformableObjectParameters.cxx:34; OrientedSurfaceMesh.cxx:247-290 runs its
    normals filter with consistency, automatic outward orientation and flipping on).

    The filter (myvtkPolyDataNormals.cxx:209-290 and 549-617): take the left-most point (smallest
    x) that has unvisited triangles; among those triangles pick the one whose normal
    ((v3 - v2) x (v1 - v2) / 2 on the original ordering) has the largest |x| component and reverse
    it when that normal points to +x, exclusive-or `flip`; then visit the mesh breadth first from
    it, reversing every edge neighbour (a triangle sharing exactly one edge owner) whose ordering
    runs the shared edge in the same direction. Repeat for every connected component. Reversing a
    triangle reverses its vertex order."""
    tris = [list(t) for t in np.asarray(tris)]
    old = [tuple(t) for t in tris]
    n = len(tris)
    cells_of: dict[int, list[int]] = {}
    for c, t in enumerate(old):
        for v in t:
            cells_of.setdefault(int(v), []).append(c)

    def edge_neighbors(c, a, b):
        return [k for k in cells_of.get(int(a), []) if k != c and b in old[k]]

    visited = [False] * n
    order = sorted(range(len(pts)), key=lambda i: (pts[i][0], i))  # priority queue by x
    qi = 0
    while qi < len(order):
        seed, best, reverse = -1, 0.0, False
        while qi < len(order) and seed < 0:
            pid = order[qi]
            qi += 1
            for c in cells_of.get(pid, []):
                if visited[c]:
                    continue
                v1, v2, v3 = (np.asarray(pts[i], dtype=np.float64) for i in old[c])
                a, b = v3 - v2, v1 - v2
                nx = (a[1] * b[2] - a[2] * b[1]) / 2.0
                if abs(nx) > best:
                    best, seed, reverse = abs(nx), c, nx > 0
        if seed < 0:
            break
        if reverse != flip:
            tris[seed].reverse()
        visited[seed] = True
        wave = [seed]
        while wave:
            nxt = []
            for c in wave:
                t = tris[c]
                for j in range(3):
                    p1, p2 = t[j], t[(j + 1) % 3]
                    nb = edge_neighbors(c, p1, p2)
                    if len(nb) != 1 or visited[nb[0]]:
                        continue
                    k = nb[0]
                    u = tris[k]
                    l = u.index(p2)
                    if u[(l + 1) % 3] != p1:
                        u.reverse()
                    visited[k] = True
                    nxt.append(k)
            wave = nxt
    return np.array(tris, dtype=np.int32)


def _archive_items(text: str):
    """Items of a Boost text archive in file order: ("blob", bytes) for base64 runs, ("tok", str)
    for every other token."""
    items = []
    blob = []
    for line in text.split("\n"):
        s = line.strip()
        # a blob starts on a base64 line of 16+ characters or a padded one, and runs on over the
        # following base64 lines (its last line can be short)
        if s and _B64.fullmatch(s) and not s.isdigit() and (blob or len(s) >= 16 or s.endswith("=")):
            blob.append(s)
            continue
        if blob:
            items.append(("blob", base64.b64decode("".join(blob))))
            blob = []
        items.extend(("tok", t) for t in s.split())
    if blob:
        items.append(("blob", base64.b64decode("".join(blob))))
    return items


def read_state_blobs(path: str):
    """Every matrix and vector of a DeformationState archive in file order, as dicts with keys
    `name` (the map key written before it, or None), `shape`, `value` (float64, shaped, matrices
    converted from column-major) and `index` (position within a matrix list: the matrices of one
    fixed or random effect, e.g. one per template object or per subject, follow the key that
    names the first one). Also returns the scalar tokens that precede the first blob."""
    with open(path) as f:
        items = _archive_items(f.read())
    out = []
    toks: list[str] = []
    head = None
    for kind, v in items:
        if kind == "tok":
            toks.append(v)
            continue
        if head is None:
            head = list(toks)
        a = np.frombuffer(v, dtype="<f8").copy()
        name = None
        for k in range(len(toks) - 1, 0, -1):  # a length-prefixed key: "<len> <name>"
            if (toks[k - 1].isdigit() and int(toks[k - 1]) == len(toks[k])
                    and re.fullmatch(r"[A-Za-z_][A-Za-z0-9_]*", toks[k])):
                name = toks[k]
                break
        ints = [int(t) for t in toks if t.lstrip("-").isdigit()]
        shaped = len(ints) >= 2 and ints[-2] * ints[-1] == a.size and ints[-1] > 0
        prev = out[-1] if out else None
        if shaped and name is not None:
            r, c = ints[-2], ints[-1]
            out.append({"name": name, "shape": (r, c), "value": a.reshape(c, r).T.copy(), "index": 0})
        elif shaped and prev is not None and len(prev["shape"]) == 2 and prev["name"] is not None:
            r, c = ints[-2], ints[-1]  # the next matrix of the same list
            out.append({"name": prev["name"], "shape": (r, c), "value": a.reshape(c, r).T.copy(),
                        "index": prev["index"] + 1})
        else:
            out.append({"name": name, "shape": (a.size,), "value": a, "index": 0})
        toks = []
    return out, head or toks


def read_deformation_state(path: str):
    """The final FastGradientAscent state (FastGradientAscent.cxx:313-322) of a landmark
    registration or deterministic atlas: fields iter, freeze_counter, tau (scalars), step,
    grad_sq_norms (vectors), control_points, template (fixed effects), aux_control_points,
    aux_template, the control-point gradient (grad_control_points), grad_template, momenta,
    aux_momenta, the momenta gradient, and history (one [data, regularity] row per iteration).
    A multi-object template is a list of matrices (one per object); the momenta of several
    subjects stack to (subjects, control points, d)."""
    blobs, head = read_state_blobs(path)

    def is_float(t):
        try:
            float(t)
        except ValueError:
            return False
        return not t.lstrip("-").isdigit()

    tau_i = next((i for i, t in enumerate(head) if is_float(t)), None)
    st: dict = {}
    if tau_i is not None:
        st["tau"] = float(head[tau_i])
        uints = [int(t) for t in head[:tau_i] if t.isdigit()]
        # ... <count=2> <item_version> <iter> <freeze> <class info> <count=1> <item_version> tau
        st["iter"], st["freeze_counter"] = uints[-6], uints[-5]
    vecs = [b for b in blobs if b["name"] is None]
    named = [b for b in blobs if b["name"] is not None]
    st["step"], st["grad_sq_norms"] = vecs[0]["value"], vecs[1]["value"]
    st["history"] = np.stack([b["value"] for b in vecs[2:]])
    groups: dict[str, list] = {}  # per name: one list of matrices per written effect map
    for b in named:
        g = groups.setdefault(b["name"], [])
        if b["index"] == 0:
            g.append([])
        g[-1].append(b["value"])
    # a one-matrix list is that matrix; same-shaped lists (one per subject) stack; others stay lists
    by_name = {k: [m[0] if len(m) == 1 else (np.stack(m) if len({x.shape for x in m}) == 1 and k == "Momenta"
                                              else m) for m in v] for k, v in groups.items()}
    cps, tds, moms = by_name.get("ControlPoints", []), by_name.get("TemplateData", []), by_name.get("Momenta", [])
    st["control_points"], st["aux_control_points"] = cps[0], cps[1]
    if len(cps) > 2:
        st["grad_control_points"] = cps[2]
    if tds:
        st["template"], st["aux_template"] = tds[0], tds[1]
        if len(tds) > 2:
            st["grad_template"] = tds[2]
    st["momenta"], st["aux_momenta"], st["grad_momenta"] = moms[0], moms[1], moms[2]
    return st
