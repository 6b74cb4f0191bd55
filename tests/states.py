"""Seeded random element states in the packed 96-double record layout."""
import numpy as np
from scipy.spatial.transform import Rotation as Rot

import oracle as O


def beam_states(n, seed=0, angle=0.3, small=False, damping=(0.0, 0.01)):
    rng = np.random.default_rng(seed)
    inp = np.zeros((n, 96))
    for e in range(n):
        l0 = rng.uniform(0.5, 2.0)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        X1 = rng.normal(size=3)
        X2 = X1 + l0 * d
        Re0 = O.get_Re0(X1[None], X2[None])[0]
        a = angle * (1e-6 if small else 1.0)
        R1 = Rot.from_rotvec(rng.normal(size=3) * a).as_matrix()
        R2 = Rot.from_rotvec(rng.normal(size=3) * a).as_matrix()
        dR1 = Rot.from_rotvec(rng.normal(size=3) * a * 0.1).as_matrix()
        dR2 = Rot.from_rotvec(rng.normal(size=3) * a * 0.1).as_matrix()
        E = rng.uniform(1e5, 1e7)
        rho = rng.uniform(1, 10)
        r = rng.uniform(0.01, 0.1) * l0
        Kb, Jr, Ar = O.beam_constants(E, 0.3, rho, r, np.array([l0]))
        p = inp[e]
        p[0:3], p[3:6] = X1, X2
        p[6:9] = rng.normal(size=3) * 0.05 * l0
        p[9:12] = rng.normal(size=3) * 0.05 * l0
        p[12:21], p[21:30] = R1.flatten("F"), R2.flatten("F")
        p[30:39], p[39:48] = dR1.flatten("F"), dR2.flatten("F")
        p[48:72] = rng.normal(size=24)
        p[72] = l0
        p[73:82] = Re0
        p[82] = Kb[0, 0]
        p[83:89] = Kb[0, 1:]
        p[89:92] = Jr[0]
        p[92] = Ar[0]
        p[93] = rng.choice(damping)
        p[94] = r
    return inp


def contact_states(n, center, Rs, rb, seed=1):
    """Elements placed across a sphere surface so that most Gauss points touch."""
    rng = np.random.default_rng(seed)
    inp = np.zeros((n, 96))
    for e in range(n):
        l0 = rng.uniform(0.5, 1.0) * rb * 20
        dirn = rng.normal(size=3)
        dirn /= np.linalg.norm(dirn)
        mid = center + dirn * (Rs + rb * rng.uniform(-0.5, 1.2))
        t = np.cross(dirn, rng.normal(size=3))
        t /= np.linalg.norm(t)
        X1, X2 = mid - 0.5 * l0 * t, mid + 0.5 * l0 * t
        p = inp[e]
        p[0:3], p[3:6] = X1, X2
        p[6:9] = rng.normal(size=3) * 0.02 * rb
        p[9:12] = rng.normal(size=3) * 0.02 * rb
        p[12:21] = Rot.from_rotvec(rng.normal(size=3) * 0.2).as_matrix().flatten("F")
        p[21:30] = Rot.from_rotvec(rng.normal(size=3) * 0.2).as_matrix().flatten("F")
        p[30:39] = Rot.from_rotvec(rng.normal(size=3) * 0.02).as_matrix().flatten("F")
        p[39:48] = Rot.from_rotvec(rng.normal(size=3) * 0.02).as_matrix().flatten("F")
        p[48:60] = rng.normal(size=12) * 0.1
        p[72] = l0
        p[73:82] = O.get_Re0(X1[None], X2[None])[0]
        p[94] = rb
    return inp


def plane_states(n, axis, position, rb, seed=2, spread=0.2):
    """Elements lying across the plane x[axis] = position (within ±spread in the plane),
    tilted slightly out of it, so that most Gauss points touch."""
    rng = np.random.default_rng(seed)
    normal = np.zeros(3)
    normal[axis] = 1.0
    inp = contact_states(n, np.zeros(3), 1.0, rb, seed=seed)
    for e in range(n):
        p = inp[e]
        l0 = p[72]
        mid = rng.uniform(-spread, spread, 3)
        mid[axis] = position + rb * rng.uniform(-0.5, 1.2)
        t = rng.normal(size=3)
        t[axis] = 0.0
        t /= np.linalg.norm(t)
        t = t + normal * rng.uniform(-0.05, 0.05)
        t /= np.linalg.norm(t)
        X1, X2 = mid - 0.5 * l0 * t, mid + 0.5 * l0 * t
        p[0:3], p[3:6] = X1, X2
        p[73:82] = O.get_Re0(X1[None], X2[None])[0]
    return inp


def rel_err(a, b, floor=1e-300):
    """Per-row normwise relative error ‖a-b‖/‖b‖."""
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), floor)
