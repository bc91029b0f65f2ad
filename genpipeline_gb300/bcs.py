"""Boundary conditions and load cases (host logic, numpy).

Every function returns ``(f, fixed_dofs)``: ``f`` the FP64 load vector of length
3*(nx+1)*(ny+1)*(nz+1) and ``fixed_dofs`` the sorted unique fixed DOF indices. ``node_mask``
turns the fixed list into the device format (one byte per node, bit c = DOF 3n+c fixed).

* ``reference_cpu``   -- ``SIMPSolver._get_bcs`` / ``_get_face_mask``
                         (genpipeline/topology/simp_solver.py:81-175)
* ``reference_gpu``   -- ``SIMPSolverGPU._get_bcs`` with its multi-position and grid loads
                         (genpipeline/topology/simp_solver_gpu.py:138-311)
* ``reference_dense`` -- ``DenseGPUSolver._get_bcs`` (simp_solver_dense_gpu.py:209-236)
* ``cantilever_tip``, ``top_patch``, ``torsion_couple``, ``edge_line_load`` -- the load cases
  of the benchmark configurations (point load at (nx, ny//2, 0) with x=0 clamped; uniform
  traction on the central patch of the top face with z=0 clamped; a unit torque couple on
  the x=nx face with x=0 clamped; a line load along the bottom edge of the x=nx face).
"""
from __future__ import annotations

import numpy as np

_FACES = ("x_min", "x_max", "y_min", "y_max", "z_min", "z_max")


def n_nodes(nx, ny, nz) -> int:
    return (nx + 1) * (ny + 1) * (nz + 1)


def node_id(i, j, k, ny, nz):
    return (np.asarray(i) * (ny + 1) + np.asarray(j)) * (nz + 1) + np.asarray(k)


def _grid(nx, ny, nz):
    return np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")


def _ids(nx, ny, nz, mask):
    ix, iy, iz = _grid(nx, ny, nz)
    return ((ix * (ny + 1) + iy) * (nz + 1) + iz)[mask]


def _face_cpu(face, ix, iy, iz, nx, ny, nz):
    """simp_solver.py:159-175 -- an unknown name selects the x_max face."""
    if face == "x_min":
        return ix == 0
    if face == "x_max":
        return ix == nx
    if face == "y_min":
        return iy == 0
    if face == "y_max":
        return iy == ny
    if face == "z_min":
        return iz == 0
    if face == "z_max":
        return iz == nz
    return ix == nx


def _fixed_dofs(nodes):
    nodes = np.asarray(nodes, dtype=np.int64)
    return np.unique(np.concatenate([3 * nodes, 3 * nodes + 1, 3 * nodes + 2]))


def reference_cpu(nx, ny, nz, bcs=None, force_mag=1.0):
    """Fixed DOFs and load vector of SIMPSolver._get_bcs (simp_solver.py:81-157)."""
    b = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
    if bcs:
        b.update(bcs)
    ix, iy, iz = _grid(nx, ny, nz)
    ids = (ix * (ny + 1) + iy) * (nz + 1) + iz
    ff = b.get("fixed_face", "x_min")
    faces = ff if isinstance(ff, list) else [ff]
    fixed_nodes = np.unique(np.concatenate([ids[_face_cpu(f, ix, iy, iz, nx, ny, nz)] for f in faces]))
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    lf = b.get("load_face", "x_max")
    ld = b.get("load_dof", 2)
    multi = b.get("multi_load", False)

    def valid(mask):
        nodes = ids[mask]
        return nodes, nodes[~np.isin(nodes, fixed_nodes)]

    if multi and isinstance(ld, list):
        for d in ld:
            _, v = valid(_face_cpu(lf, ix, iy, iz, nx, ny, nz))
            if len(v) > 0:
                sel = v[::3]
                for node in sel:
                    f[3 * node + d] -= force_mag / len(sel)
    elif lf in ("center", "center_z"):
        dist = np.sqrt((ix - nx // 2) ** 2 + (iy - ny // 2) ** 2 + (iz - nz // 2) ** 2)
        _, v = valid(dist <= 2)
        if len(v) > 0:
            sel = v[::2]
            for node in sel:
                f[3 * node + ld] -= force_mag / len(sel)
    elif lf == "top":
        _, v = valid(iz == nz)
        if len(v) > 0:
            f[3 * v[len(v) // 2] + ld] = -force_mag
    elif lf == "x_max_offset":
        _, v = valid((ix == nx) & (iy >= ny // 3) & (iy <= 2 * ny // 3))
        if len(v) > 0:
            f[3 * v[len(v) // 2] + ld] = -force_mag
    else:
        nodes, v = valid(_face_cpu(lf, ix, iy, iz, nx, ny, nz))
        mid = v[len(v) // 2] if len(v) > 0 else nodes[len(nodes) // 2]
        f[3 * mid + ld] = -force_mag
    return f, _fixed_dofs(fixed_nodes)


def _face_gpu_fixed(ff, ix, iy, iz, nx, ny, nz):
    """simp_solver_gpu.py:147-162 -- a list or unknown name selects the x_min face."""
    table = {"x_min": ix == 0, "x_max": ix == nx, "y_min": iy == 0, "y_max": iy == ny,
             "z_min": iz == 0, "z_max": iz == nz}
    return table.get(ff, ix == 0) if isinstance(ff, str) else ix == 0


def _face_gpu_load(lf, ix, iy, iz, nx, ny, nz):
    """simp_solver_gpu.py:170-185 -- an unknown name selects the x_max face."""
    table = {"x_max": ix == nx, "x_min": ix == 0, "y_max": iy == ny, "y_min": iy == 0,
             "z_max": iz == nz, "z_min": iz == 0}
    return table.get(lf, ix == nx) if isinstance(lf, str) else ix == nx


def _gpu_pattern_load(nx, ny, nz, b, force_mag, fixed_nodes):
    """The named-position and grid loads of SIMPSolverGPU (simp_solver_gpu.py:250-311)."""
    ix, iy, iz = _grid(nx, ny, nz)
    ids = (ix * (ny + 1) + iy) * (nz + 1) + iz
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    ld = b.get("load_dof", 2)
    positions = b.get("load_positions", None)
    if positions:
        # _apply_multi_position_load (:250-292): position masks over the whole grid.
        for pos in positions:
            if pos == "top":
                m = iz == nz
            elif pos == "bottom":
                m = iz == 0
            elif pos in ("mid", "mid_z"):
                m = (iz >= nz // 3) & (iz <= 2 * nz // 3)
            elif pos == "mid_y":
                m = (iy >= ny // 3) & (iy <= 2 * ny // 3)
            else:
                m = iz == nz // 2
            nodes = ids[m]
            v = nodes[~np.isin(nodes, fixed_nodes)]
            if len(v) > 0:
                fpn = float(force_mag) / len(positions)
                for node in v[:: max(1, len(v) // 3)]:
                    f[3 * node + ld] -= fpn
        return f
    # _apply_grid_load (:294-311): rows of constant z every max(1, nz//4).
    spacing = max(1, nz // 4)
    for zv in range(0, nz + 1, spacing):
        nodes = ids[iz == zv]
        v = nodes[~np.isin(nodes, fixed_nodes)]
        if len(v) > 0:
            fpn = float(force_mag) / ((nz // spacing) + 1)
            for node in v[:: max(1, len(v) // 2)]:
                f[3 * node + ld] -= fpn
    return f


def generator(nx, ny, nz, bcs=None, force_mag=1.0):
    """Boundary conditions of the data generator's geometries (topo_data_gen.py:41-95): the
    clamped faces and loads of SIMPSolver._get_bcs (simp_solver.py:81-157), which accepts
    lists of faces and of load directions; a named-position or grid load (multi_load with
    load_positions / load_pattern), which only SIMPSolverGPU implements
    (simp_solver_gpu.py:250-311), is spread as that class spreads it, over the nodes that the
    clamped faces leave free."""
    b = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
    if bcs:
        b.update(bcs)
    f, fixed = reference_cpu(nx, ny, nz, b, force_mag)
    if b.get("multi_load") and (b.get("load_positions") or b.get("load_pattern") == "grid"):
        f = _gpu_pattern_load(nx, ny, nz, b, force_mag, np.unique(fixed // 3))
    return f, fixed


def reference_gpu(nx, ny, nz, bcs=None, force_mag=1.0):
    """Fixed DOFs and load vector of SIMPSolverGPU._get_bcs (simp_solver_gpu.py:138-311)."""
    b = {"fixed_face": "x_min", "load_face": "x_max", "load_dof": 2}
    if bcs:
        b.update(bcs)
    ix, iy, iz = _grid(nx, ny, nz)
    ids = (ix * (ny + 1) + iy) * (nz + 1) + iz
    fixed_nodes = ids[_face_gpu_fixed(b.get("fixed_face", "x_min"), ix, iy, iz, nx, ny, nz)]
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    lf = b.get("load_face", "x_max")
    ld = b.get("load_dof", 2)
    multi = b.get("multi_load", False)
    if multi and (b.get("load_positions") or b.get("load_pattern") == "grid"):
        return _gpu_pattern_load(nx, ny, nz, b, force_mag, fixed_nodes), _fixed_dofs(fixed_nodes)
    nodes = ids[_face_gpu_load(lf, ix, iy, iz, nx, ny, nz)]
    if len(nodes) > 0:
        v = nodes[~np.isin(nodes, fixed_nodes)]
        if len(v) == 0:
            v = nodes
        f[3 * v + ld] = -float(force_mag) / len(v)
    return f, _fixed_dofs(fixed_nodes)


def reference_dense(nx, ny, nz, force_mag=1000.0):
    """DenseGPUSolver._get_bcs (simp_solver_dense_gpu.py:209-236): x_min, y_min and z_min
    faces fixed; -z load spread over every node of the x_max face."""
    ix, iy, iz = _grid(nx, ny, nz)
    ids = (ix * (ny + 1) + iy) * (nz + 1) + iz
    fixed_nodes = ids[(ix == 0) | (iy == 0) | (iz == 0)]
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    load = ids[ix == nx]
    f[3 * load + 2] = -float(force_mag) / len(load)
    return f, _fixed_dofs(fixed_nodes)


# ---- load cases of the benchmark configurations -------------------------------------------
def clamp_face(nx, ny, nz, face):
    ix, iy, iz = _grid(nx, ny, nz)
    return _fixed_dofs(_ids(nx, ny, nz, _face_cpu(face, ix, iy, iz, nx, ny, nz)))


def cantilever_tip(nx, ny, nz, force=1.0):
    """x=0 clamped; unit -z point load at node (nx, ny//2, 0) (mid-bottom of the x=nx face)."""
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    f[3 * int(node_id(nx, ny // 2, 0, ny, nz)) + 2] = -force
    return f, clamp_face(nx, ny, nz, "x_min")


def top_patch(nx, ny, nz, force=1.0, frac=0.25):
    """z=0 clamped; uniform -z traction of total ``force`` on the central frac*nx x frac*ny
    element patch of the z=nz face, as consistent nodal loads (each loaded quad gives a
    quarter of its share to each of its 4 nodes)."""
    px, py = max(1, int(round(nx * frac))), max(1, int(round(ny * frac)))
    i0, j0 = (nx - px) // 2, (ny - py) // 2
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    per = force / (px * py) / 4.0
    for i in range(i0, i0 + px):
        for j in range(j0, j0 + py):
            for di in (0, 1):
                for dj in (0, 1):
                    f[3 * int(node_id(i + di, j + dj, nz, ny, nz)) + 2] -= per
    return f, clamp_face(nx, ny, nz, "z_min")


def torsion_couple(nx, ny, nz, torque=1.0):
    """x=0 clamped; on every node of the x=nx face a force t x (r - c) in the y-z plane
    (t = x axis, c = face centre), scaled to a total torque ``torque`` about x; the net
    force is zero by symmetry."""
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    jj, kk = np.meshgrid(np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    yc, zc = ny / 2.0, nz / 2.0
    ry, rz = (jj - yc).ravel(), (kk - zc).ravel()
    fy, fz = -rz, ry
    s = torque / float(np.sum(ry * fz - rz * fy))
    nodes = node_id(nx, jj.ravel(), kk.ravel(), ny, nz)
    f[3 * nodes + 1] += s * fy
    f[3 * nodes + 2] += s * fz
    return f, clamp_face(nx, ny, nz, "x_min")


def edge_line_load(nx, ny, nz, force=1.0):
    """x=0 clamped; -z line load of total ``force`` along the bottom edge of the x=nx face,
    nodes (nx, j, 0), j = 0..ny, end nodes at half weight."""
    f = np.zeros(3 * n_nodes(nx, ny, nz))
    w = np.full(ny + 1, 1.0)
    w[0] = w[-1] = 0.5
    w *= force / w.sum()
    nodes = node_id(nx, np.arange(ny + 1), 0, ny, nz)
    f[3 * nodes + 2] -= w
    return f, clamp_face(nx, ny, nz, "x_min")


LOAD_CASES = {"cantilever": cantilever_tip, "top_patch": top_patch, "torsion": torsion_couple,
              "edge_line": edge_line_load}


def node_mask(nx, ny, nz, fixed_dofs) -> np.ndarray:
    """One byte per node; bit c set when DOF 3n+c is fixed."""
    m = np.zeros(n_nodes(nx, ny, nz), dtype=np.uint8)
    d = np.asarray(fixed_dofs, dtype=np.int64)
    np.bitwise_or.at(m, d // 3, (1 << (d % 3)).astype(np.uint8))
    return m


def dof_mask(nx, ny, nz, fixed_dofs) -> np.ndarray:
    """One byte per DOF (1 = fixed), the oracle's format."""
    m = np.zeros(3 * n_nodes(nx, ny, nz), dtype=np.uint8)
    m[np.asarray(fixed_dofs, dtype=np.int64)] = 1
    return m
