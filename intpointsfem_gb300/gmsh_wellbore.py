"""Gmsh 4.1 files of the reference's wellbore meshes.

The reference generates its meshes with Gmsh from gmsh/wellbore.geo: a full
annulus (well radius 0.1, outer radius 4) split into four quadrant surfaces,
every quarter circle and radial line a transfinite line of n nodes, the radial
lines graded with "Using Progression q", the surfaces transfinite and
recombined into quadrilaterals.  Its shipped meshes are n = 32, q = 1.175
(wellbore_1.msh) and n = 64, q = 1.075 (wellbore_2.msh); the .geo lists
128/1.04, 256/1.0175 and 512/1.009 for the larger meshes of its logs, whose
files are not part of the reference.

Transfinite interpolation between two concentric arcs and two radial lines
with the same node distribution puts every node on the circle of its radial
index, at its arc's angle, so the mesh is the polar grid written here.  The
radial nodes follow the geometric progression t_i = (q^i - 1)/(q^(n-1) - 1);
Gmsh evaluates the same distribution by numerical integration, so its
coordinates differ from these in the eighth digit.

Physical names and tags are those of wellbore.geo and of the reference's
files: Omega (2, 1), bc_wellbore (1, 2), bc_farfield (1, 3), fixed_x (0, 4)
at (0, +-r_out), fixed_y (0, 5) at (+-r_out, 0).
"""
import math

import numpy as np

# (nodes per line, radial progression) of the reference's meshes 1-5
REFERENCE_MESHES = {1: (32, 1.175), 2: (64, 1.075), 3: (128, 1.04), 4: (256, 1.0175), 5: (512, 1.009)}


def wellbore_nodes(n, q, r_in=0.1, r_out=4.0):
    """(radii[n], angles[4(n-1)]) of the polar grid"""
    i = np.arange(n, dtype=np.float64)
    t = (q ** i - 1.0) / (q ** (n - 1) - 1.0) if q != 1.0 else i / (n - 1)
    r = r_in + (r_out - r_in) * t
    r[0], r[-1] = r_in, r_out
    m = 4 * (n - 1)
    th = np.array([(k // (n - 1)) * (math.pi / 2) + (k % (n - 1)) * (math.pi / 2) / (n - 1) for k in range(m)])
    return r, th


def write_wellbore_msh(path, n, q, r_in=0.1, r_out=4.0, tri_quadrants=()):
    """Write the wellbore mesh with n nodes per quarter arc and radial line and
    radial progression q as a Gmsh 4.1 ASCII file; returns (n_nodes, n_elements).
    The quadrants listed in tri_quadrants (0-3) are split into triangles (each
    quadrilateral along its diagonal from its first vertex), as wellbore.geo
    leaves the surfaces it does not recombine."""
    if n < 2:
        raise ValueError("n must be at least 2")
    r, th = wellbore_nodes(n, q, r_in, r_out)
    m = 4 * (n - 1)

    def tag(i, k):                     # node tag of radial index i, angular index k (1-based tags)
        return 1 + i * m + (k % m)

    xy = np.zeros((n * m, 2))
    for i in range(n):
        xy[i * m:(i + 1) * m, 0] = r[i] * np.cos(th)
        xy[i * m:(i + 1) * m, 1] = r[i] * np.sin(th)
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$PhysicalNames", "5",
             '0 4 "fixed_x"', '0 5 "fixed_y"', '1 2 "bc_wellbore"', '1 3 "bc_farfield"', '2 1 "Omega"',
             "$EndPhysicalNames", "$Entities", "8 12 4 0"]
    # points 1-4 on the well (no tag), 5-8 on the outer circle at 0, 90, 180, 270 degrees
    for p in range(4):
        lines.append("%d %.17g %.17g 0 0" % (p + 1, r_in * math.cos(p * math.pi / 2), r_in * math.sin(p * math.pi / 2)))
    for p in range(4):
        lines.append("%d %.17g %.17g 0 1 %d" % (p + 5, r_out * math.cos(p * math.pi / 2),
                                                r_out * math.sin(p * math.pi / 2), 5 if p % 2 == 0 else 4))
    # curves 1-4 well arcs (tag 2), 5-8 outer arcs (tag 3), 9-12 radial lines (no tag)
    for c in range(4):
        lines.append("%d %.17g %.17g 0 %.17g %.17g 0 1 2 2 %d -%d" % (c + 1, -r_in, -r_in, r_in, r_in, c + 1,
                                                                       (c + 1) % 4 + 1))
    for c in range(4):
        lines.append("%d %.17g %.17g 0 %.17g %.17g 0 1 3 2 %d -%d" % (c + 5, -r_out, -r_out, r_out, r_out, c + 5,
                                                                       (c + 1) % 4 + 5))
    for c in range(4):
        lines.append("%d %.17g %.17g 0 %.17g %.17g 0 0 2 %d -%d" % (c + 9, -r_out, -r_out, r_out, r_out, c + 1,
                                                                     c + 5))
    for s in range(4):
        lines.append("%d %.17g %.17g 0 %.17g %.17g 0 1 1 4 %d %d %d %d" % (s + 1, -r_out, -r_out, r_out, r_out,
                                                                            -(s + 1), s + 9, s + 5,
                                                                            -((s + 1) % 4 + 9)))
    lines.append("$EndEntities")
    # nodes: one block on surface 1 (entity assignment has no bearing on the mesh)
    nn = n * m
    lines += ["$Nodes", "1 %d 1 %d" % (nn, nn), "2 1 0 %d" % nn]
    lines += [str(k + 1) for k in range(nn)]
    lines += ["%.17g %.17g 0" % (x, y) for x, y in xy]
    lines.append("$EndNodes")
    # elements: the 4 tagged points, the well and outer arcs, the quadrilaterals per quadrant
    blocks = []
    eid = 1
    for p in range(4):
        blocks.append(("0 %d 15 1" % (p + 5), ["%d %d" % (eid, tag(n - 1, p * (n - 1)))]))
        eid += 1
    for c, i in ((0, 0), (1, n - 1)):
        for quad in range(4):
            rows = []
            for k in range(quad * (n - 1), (quad + 1) * (n - 1)):
                rows.append("%d %d %d" % (eid, tag(i, k), tag(i, k + 1)))
                eid += 1
            blocks.append(("1 %d 1 %d" % (quad + 1 + 4 * c, len(rows)), rows))
    nq = 0
    for quad in range(4):
        rows = []
        tri = quad in tri_quadrants
        for j in range(n - 1):                       # radial layer
            for k in range(quad * (n - 1), (quad + 1) * (n - 1)):
                v = (tag(j, k), tag(j + 1, k), tag(j + 1, k + 1), tag(j, k + 1))
                if tri:
                    rows.append("%d %d %d %d" % (eid, v[0], v[1], v[2]))
                    rows.append("%d %d %d %d" % (eid + 1, v[0], v[2], v[3]))
                    eid += 2
                else:
                    rows.append("%d %d %d %d %d" % (eid, v[0], v[1], v[2], v[3]))
                    eid += 1
        nq += len(rows)
        blocks.append(("2 %d %d %d" % (quad + 1, 2 if tri else 3, len(rows)), rows))
    lines += ["$Elements", "%d %d 1 %d" % (len(blocks), eid - 1, eid - 1)]
    for head, rows in blocks:
        lines.append(head)
        lines += rows
    lines.append("$EndElements")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return nn, nq


def reference_bcs(cohesion=5.0):
    """Material and boundary data of the reference's verification configuration
    (WellboreConfigRK, main.cpp:397-446): E 2000, nu 0.2, c 5 (1e10 for the
    elastic case), phi = psi = 20 deg; well normal stress -(-40 - (-50)) = -10,
    outer normal stress -(-50 - (-50)) - 0.00625, u_x = 0 at fixed_x, u_y = 0 at
    fixed_y.  Returns (bcs, material keyword arguments) for GmshProblem."""
    bcs = [("bc_wellbore", 6, -1.0 * (-40.0 - (-50.0))), ("bc_farfield", 6, -1.0 * (-50.0 - (-50.0)) - 0.00625),
           ("fixed_x", 3, 1.0, 0.0), ("fixed_y", 3, 0.0, 1.0)]
    return bcs, dict(E=2000.0, nu=0.2, cohesion=cohesion, phi_deg=20.0, psi_deg=20.0)
