"""Write rational Bezier patches as an IGES file (entity 128, rational
B-spline surface) in the fixed 80-column layout the geometry reader expects:
section letter in column 73, sequence number in columns 74-80, two directory
lines per entity, parameter data in columns 1-64 with the directory pointer in
65-72. Used by the tests to produce IGES inputs from the .dat geometries.
"""


def read_dat(path):
    """Patches of an Octave-NURBS .dat file: list of (px, py, X, Y, Z, W) with
    px, py control points per direction and the homogeneous coordinate
    matrices flattened first-index-fastest."""
    with open(path) as f:
        lines = f.read().splitlines()
    npatch = int(lines[4].split()[2])
    out, k = [], 5
    for _ in range(npatch):
        deg = [int(v) for v in lines[k + 1].split()]
        ncp = [int(v) for v in lines[k + 2].split()]
        mats = [[float(v) for v in lines[k + 5 + c].split()] for c in range(4)]
        out.append((ncp[0], ncp[1], *mats))
        k += 9
        assert deg[0] + 1 == ncp[0] and deg[1] + 1 == ncp[1]
    return out


def _fmt(v):
    return repr(float(v))


def write_igs(patches, path, knots=None, entity=128):
    """patches: (px, py, X, Y, Z, W) with homogeneous X, Y, Z (as in .dat);
    knots: optional per-patch (knots_s, knots_t) overriding the Bezier ones."""
    start = ["Bezier patches written as IGES entity 128"]
    glob = ["1H,,1H;,4Hgeom,4Hgeom,4Hgeom,4Hgeom,32,38,6,308,15,4Hgeom,1.,2,2HMM,1,0.1,13H000000.000000,"
            "1E-6,1.,1H ,1H ,11,0,13H000000.000000;"]
    params = []  # (lines of one entity)
    for i, (px, py, X, Y, Z, W) in enumerate(patches):
        ks = [0.0] * px + [1.0] * px
        kt = [0.0] * py + [1.0] * py
        if knots is not None:
            ks, kt = knots[i]
        m1, m2 = px - 1, py - 1
        k1, k2 = len(ks) - m1 - 2, len(kt) - m2 - 2
        vals = [entity, k1, k2, m1, m2, 0, 0, 1, 0, 0] + ks + kt
        n = (k1 + 1) * (k2 + 1)
        if knots is not None:
            W = [1.0] * n
            X = Y = Z = [0.5] * n
        vals += list(W[:n])
        for q in range(n):
            vals += [X[q] / W[q], Y[q] / W[q], Z[q] / W[q]]
        vals += [0.0, 1.0, 0.0, 1.0]
        toks = [str(v) if isinstance(v, int) else _fmt(v) for v in vals]
        lines, cur = [], ""
        for j, t in enumerate(toks):
            t += ";" if j == len(toks) - 1 else ","
            if len(cur) + len(t) > 64:
                lines.append(cur)
                cur = ""
            cur += t
        lines.append(cur)
        params.append(lines)
    out = []
    for j, l in enumerate(start):
        out.append("%-72sS%7d" % (l, j + 1))
    for j, l in enumerate(glob):
        out.append("%-72sG%7d" % (l, j + 1))
    seq, first = 1, 1
    for i, lines in enumerate(params):
        de = 2 * i + 1
        out.append("%8d%8d%8d%8d%8d%8d%8d%8d%8sD%7d" % (entity, first, 0, 0, 0, 0, 0, 0, "00000000", de))
        out.append("%8d%8d%8d%8d%8d%8s%8s%8s%8sD%7d" % (entity, 0, 0, len(lines), 0, "", "", "", "", de + 1))
        first += len(lines)
    pseq = 1
    for i, lines in enumerate(params):
        for l in lines:
            out.append("%-64s%8dP%7d" % (l, 2 * i + 1, pseq))
            pseq += 1
    out.append("%-72sT%7d" % ("S%7dG%7dD%7dP%7d" % (len(start), len(glob), 2 * len(params), pseq - 1), 1))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
