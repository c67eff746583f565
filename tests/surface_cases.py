"""Surface scenes shared by the CPU (oracle) and GPU surface tests."""
import numpy as np

from gpusmoldyn_gb300 import _lib as L


def tri_box(s, surface, lo, hi):
    """A closed axis-aligned box of 12 triangles, front faces outward."""
    V = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])], np.float64)
    c = V.mean(0)
    ids = []
    for q in ((0, 1, 3, 2), (4, 5, 7, 6), (0, 1, 5, 4), (2, 3, 7, 6), (0, 2, 6, 4), (1, 3, 7, 5)):
        for tri in ((q[0], q[1], q[2]), (q[0], q[2], q[3])):
            v = V[list(tri)]
            if np.dot(np.cross(v[1] - v[0], v[2] - v[0]), v[0] - c) < 0:
                v = v[[0, 2, 1]]
            ids.append(s.add_panel(surface, "tri", list(v.ravel())))
    return ids


def capped_cylinder(s, surface, x, y, z0, z1, r):
    """An open cylinder along z closed by two disks, front faces outward."""
    s.add_panel(surface, "cyl", [x, y, z0, x, y, z1, r], front=1)
    s.add_panel(surface, "disk", [x, y, z0, r, 0, 0, -1])
    s.add_panel(surface, "disk", [x, y, z1, r, 0, 0, 1])


def mixed_scene(s, A, B, C, D):
    """Every panel shape and action on one 6 um box (species A..D):
    a reflecting sphere, an absorbing-for-A plane, a triangle box that
    absorbs B from outside and reflects the rest, a capped cylinder that
    reflects C and D, a hemisphere that absorbs A on its front and reflects B
    on its back, a one-sided rectangle (front reflects, back transmits)."""
    f0 = s.add_surface()
    s.set_surface_action(f0, L.BD_ALL_SPECIES, "both", "reflect")
    s.add_panel(f0, "sph", [1.5, 1.5, 1.5, 1.0])
    f1 = s.add_surface()
    s.set_surface_action(f1, A, "both", "absorb")
    s.set_surface_action(f1, C, "both", "reflect")
    s.add_panel(f1, "rect", [5.2, 0.0, 0.0, 6.0, 6.0], axis=0, front=1)
    f2 = s.add_surface()
    s.set_surface_action(f2, L.BD_ALL_SPECIES, "both", "reflect")
    s.set_surface_action(f2, B, "front", "absorb")
    tri_box(s, f2, (3.2, 0.6, 0.6), (4.6, 2.4, 2.4))
    f3 = s.add_surface()
    s.set_surface_action(f3, C, "both", "reflect")
    s.set_surface_action(f3, D, "both", "reflect")
    capped_cylinder(s, f3, 1.5, 4.2, 0.5, 5.0, 0.9)
    f4 = s.add_surface()
    s.set_surface_action(f4, A, "front", "absorb")
    s.set_surface_action(f4, B, "back", "reflect")
    s.add_panel(f4, "hemi", [4.2, 4.2, 3.0, 1.1, 0.3, 0.2, 1.0], front=1)
    f5 = s.add_surface()
    s.set_surface_action(f5, L.BD_ALL_SPECIES, "front", "reflect")
    s.add_panel(f5, "rect", [0.0, 3.0, 0.0, 3.0, 6.0], axis=1, front=1)
    s.add_panel(f5, "rect", [0.0, 6.0, 5.5, 6.0, -2.5], axis=2, front=-1)
    return [f0, f1, f2, f3, f4, f5]
