"""Generate quadrature_tables.h from AFEPack's template-geometry files.

AFEPack integrates element matrices with tabulated quadrature rules stored in
``template/triangle/triangle.tmp_geo`` and ``template/tetrahedron/tetrahedron.tmp_geo``
(read by ``QuadratureInfoAdmin``'s stream operator, Geometry.templates.h:702-725).
Matching the reference to 1e-13 needs the very same points and weights (the
tetrahedron rules of accuracy 2 and 3 carry only eight digits), so the tables
are extracted from those files rather than recomputed.  The header is
committed; this script is rerun only when the rule set changes:

    python afepack_gb300/csrc/gen_quadrature.py <AFEPack template dir>
"""
import os
import sys

TRI_MAX_ACC = 10  # rules kept for triangles (the files go up to 20)


def tokens(path):
    out = []
    with open(path) as fh:
        for line in fh:
            out += line.split("#")[0].split()
    return out


def parse(path, dim):
    t = tokens(path)
    p = 2  # library name, volume function
    nv = int(t[p]); p += 1 + nv * dim
    for _ in range(dim + 1):
        ng = int(t[p]); p += 1
        for _ in range(ng):
            p += 1  # index
            k = int(t[p]); p += 1 + k
            k = int(t[p]); p += 1 + k
    nq = int(t[p]); p += 1
    rules = {}
    for _ in range(nq):
        acc = int(t[p]); npts = int(t[p + 1]); p += 2
        pts = []
        for _ in range(npts):
            pts.append([float(x) for x in t[p:p + dim + 1]])
            p += dim + 1
        rules[acc] = pts
    return rules


def emit(name, dim, rules, max_acc, out):
    accs = sorted(a for a in rules if a <= max_acc)
    # fallback map: a missing accuracy uses the next higher rule
    # (QuadratureInfoAdmin::find, Geometry.templates.h:672-700)
    table_of = []
    for a in range(0, max(accs) + 1):
        b = min(x for x in accs if x >= a)
        table_of.append(accs.index(b))
    offs, flat = [], []
    for a in accs:
        offs.append(len(flat))
        flat += rules[a]
    offs.append(len(flat))
    out.append(f"// {name}: rules of accuracy {accs}; each point is {dim} local coordinates then the weight")
    out.append(f"static const int {name}_MAX_ACC = {max(accs)};")
    out.append(f"static const int {name}_RULE_OF_ACC[{len(table_of)}] = {{{', '.join(map(str, table_of))}}};")
    out.append(f"static const int {name}_OFFSET[{len(offs)}] = {{{', '.join(map(str, offs))}}};")
    out.append(f"static const double {name}_POINTS[{len(flat)}][{dim + 1}] = {{")
    for pt in flat:
        out.append("  {" + ", ".join(repr(x) for x in pt) + "},")
    out.append("};")


def main():
    if len(sys.argv) > 1:
        tdir = sys.argv[1]
    else:
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "oracle"))
        import refpath
        tdir = refpath.template_dir()
        if tdir is None:
            sys.exit("AFEPack sources not found: set AFEPACK_SOURCE or pass the template directory")
    tri = parse(os.path.join(tdir, "triangle", "triangle.tmp_geo"), 2)
    tet = parse(os.path.join(tdir, "tetrahedron", "tetrahedron.tmp_geo"), 3)
    out = ["// Generated by gen_quadrature.py from AFEPack's triangle.tmp_geo and",
           "// tetrahedron.tmp_geo quadrature tables.  Do not edit.",
           "#pragma once", ""]
    emit("AFP_TRI_QUAD", 2, tri, TRI_MAX_ACC, out)
    out.append("")
    emit("AFP_TET_QUAD", 3, tet, max(tet), out)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "quadrature_tables.h")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
