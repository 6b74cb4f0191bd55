"""ORACLE — test infrastructure only.

Converts a configuration object carrying the reference's field names
(nodes.X0/u/…, beams.conn/E/…, bcs.fixed_dofs, loads.concentrated_force,
RigidInteraction) into the oracle's plain-array Scene.  Duck-typed: this
module imports nothing from the product package.
"""
from __future__ import annotations

import numpy as np

import oracle as O


def scene_from_conf(conf, inter=None) -> O.Scene:
    nd, bm = conf.nodes, conf.beams
    cf = conf.loads.concentrated_force if conf.loads is not None else None
    loaded = np.zeros(0, np.int64)
    force_fn = None
    if cf is not None and len(cf.loaded_dofs):
        loaded = np.asarray(list(cf.loaded_dofs), np.int64) - 1
        force_fn = cf.force_function
    bcs = conf.bcs
    sc = O.Scene(X0=np.array(nd.X0), conn=np.array(bm.conn), E=bm.E, nu=bm.nu, rho=bm.rho, radius=bm.radius,
                 damping=bm.damping, u0=np.array(nd.u), ud0=np.array(nd.ud), udd0=np.array(nd.udd),
                 w0=np.array(nd.w), wd0=np.array(nd.wd), wdd0=np.array(nd.wdd), R0=np.array(nd.R),
                 Re0=None if bm.Re0 is None else np.array(bm.Re0),
                 fixed_dofs=np.asarray(bcs.fixed_dofs, np.int64), displaced_idx=np.asarray(bcs.displaced_indices),
                 imposed_fn=bcs.imposed_displacements_function, loaded_dofs=loaded, force_fn=force_fn)
    if inter is not None:
        m, p = inter.master, inter.properties
        sc.contact_props = (p.kn, p.mu, p.eps_t, p.eta_n)
        sc.contact_elems = np.asarray(inter.slave.contact_beams, np.int64)
        if hasattr(m, "triangles"):  # TriangulatedSurface: the oracle's own mesh-to-SDF on the same grid
            import mesh_oracle
            o, h, dims = m.grid()
            vals = mesh_oracle.sdf_from_mesh(np.asarray(m.positions, float), np.asarray(m.triangles) - 1, o, h, dims)
            vals = vals.reshape(int(dims[2]), int(dims[1]), int(dims[0]))
            sc.surface = dict(kind="sdf", field=vals if m.inside else -vals, x0=tuple(o), h=(h, h, h))
        elif hasattr(m, "axis_index"):
            sc.surface = dict(kind="plane", axis=m.axis_index, position=float(m.position))
        elif hasattr(m, "values"):
            vals = np.asarray(m.values, float)
            sc.surface = dict(kind="sdf", field=vals if m.inside else -vals, x0=m.origin, h=m.spacing,
                              interp=getattr(m, "interpolation", "quadratic"))
        else:
            sc.surface = dict(kind="sphere", center=np.asarray(m.center, float), radius=float(m.radius))
    return sc


def params_from(p) -> O.Params:
    return O.Params(alpha=p.alpha, beta=p.beta, gamma=p.gamma, initial_timestep=p.initial_timestep,
                    min_timestep=p.min_timestep, max_timestep=p.max_timestep,
                    simulation_end_time=p.simulation_end_time,
                    accelerate_after_success_it=p.accelerate_after_success_it,
                    tolerance_residual=p.tolerance_residual, tolerance_displacement=p.tolerance_displacement,
                    max_iterations=p.max_iterations)
