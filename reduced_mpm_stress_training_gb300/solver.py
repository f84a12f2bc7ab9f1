"""Drop-in for ``MPM_Simulator_WARP`` (engine_stress/mpm_solver_warp.py:24-720).

Same class name (alias), constructor, method names, keyword arguments and
error behaviour on the substep path; the work runs in libmpm_gb300.so on
the current PyTorch CUDA stream.  Differences a caller can see:

* Device buffers are owned by this object; tensors handed to the loaders
  are copied (``clone=False`` is accepted but never aliases), and the
  ``export_*`` / ``mpm_state.*`` readers return fresh tensors in the user's
  particle order (the device copy is kept sorted by grid block).
* Errors the reference meets with ``input()`` or undefined indexing (CFL
  violation :188-192, particles leaving the grid) set bits in a device
  status word, read lazily after each substep; ``on_error`` decides whether
  they raise ``MPMStatusError`` (default), warn or are ignored.  The
  reference's per-substep debug prints (:173-190) are dropped; print_norm
  works as before.
* ``initialize`` starts from F = I (the reference leaves F = 0 until
  ``load_from_sampling`` sets it to I, :149).
* ``mpm_state.particle_F_trial`` is not kept (it lives only inside G2P);
  ``particle_Jp`` and ``particle_external_force``, which the reference
  allocates and never writes, read as zeros.
* Extensions: ``set_parameters(E=, nu=, gravity=(gx,gy,gz), particle_vol=)``,
  ``load_vol_from_tensor``, ``load_F_from_tensor``, ``load_yield_from_tensor``.
* All the reference's colliders are built.  Moving ones advance on the
  device after each active substep's grid update; their host-side
  parameters are refreshed from the device when the scene is re-uploaded.
  ``set_rotation_on_disk`` raises ValueError for |normal[0]| <= 0.1 (the
  reference's axis search loops forever there) and gives v = 0 to nodes on
  the disk axis (the reference divides 0 by 0).
* The reduced sampled-quadrature substep ``p2g2p_reduced`` (:214-227) and
  ``experiment_for_C`` (:207-209) work on dense (n, n, n) grids as the
  reference's do; the reference has no setter for the sample list, so
  ``load_sample_particle_index_from_tensor`` (or assigning
  ``mpm_state.sample_particle_index_short``) sets it, and ``g2p_sample(dt)``
  launches the sample gather the reference defines but never calls
  (engine_stress/mpm_utils.py:415-471).  A particle whose base cell is outside
  the grid, or a sample index outside [0, n), sets a status bit where the
  reference would index out of bounds.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _capi as A
from . import frames as FR
from .engine import (Collider, MPMEngine, MPMStatusError, ReducedGrid, SceneParams, lame_from_E_nu,
                     material_code, dp_alpha)


def flatten2nD(index, shape_tuple):
    """Module helper of the reference (engine_stress/mpm_solver_warp.py:14-22): the
    C-order multi-index of flat position ``index`` in an array of shape ``shape_tuple``
    (the first component is not bounded by the first extent, as there)."""
    out, rest = [], int(index)
    for d in range(len(shape_tuple)):
        stride = 1
        for e in shape_tuple[d + 1:]:
            stride *= int(e)
        q, rest = divmod(rest, stride)
        out.append(q)
    return out


class _Model:
    """Readable mirror of MPMModelStruct (engine_stress/warp_utils.py:61-81)."""

    def __init__(self, sim: "MPMSimulator"):
        self._sim = sim

    def __getattr__(self, name):
        sp = self.__dict__["_sim"]._params
        table = {
            "grid_lim": sp.grid_lim, "n_grid": sp.n_grid, "grid_dim_x": sp.n_grid,
            "grid_dim_y": sp.n_grid, "grid_dim_z": sp.n_grid, "dx": sp.dx, "inv_dx": sp.inv_dx,
            "mu": sp.mu, "lam": sp.lam, "material": sp.material, "friction_angle": sp.friction_angle,
            "alpha": dp_alpha(sp.friction_angle), "hardening": sp.hardening, "xi": sp.xi,
            "gravitational_accelaration": -sp.gravity[1], "gravity": sp.gravity,
            "n_particles": sp.n_particles,
        }
        if name in table:
            return table[name]
        if name == "yield_stress":
            return self.__dict__["_sim"]._engine.export(A.FIELD_YIELD)
        raise AttributeError(name)


class _State:
    """Readers of MPMStateStruct fields (engine_stress/warp_utils.py:84-124) in user order."""

    _VEC = {"particle_x": A.FIELD_X, "particle_x_initial": A.FIELD_X_INITIAL,
            "particle_u": A.FIELD_U, "particle_v": A.FIELD_V}
    _MAT = {"particle_F": A.FIELD_F, "particle_C": A.FIELD_C, "particle_stress": A.FIELD_STRESS}
    _SCALAR = {"particle_mass": A.FIELD_MASS, "particle_vol": A.FIELD_VOL}

    def __init__(self, sim: "MPMSimulator"):
        self._sim = sim

    def __getattr__(self, name):
        sim = self.__dict__["_sim"]
        eng = sim._engine
        n = sim.n_particles
        if name in self._VEC:
            return eng.export(self._VEC[name]).reshape(n, 3)
        if name in self._MAT:
            return eng.export(self._MAT[name]).reshape(n, 3, 3)
        if name in self._SCALAR:
            return eng.export(self._SCALAR[name])
        if name == "particle_F_disp":
            return sim._f_disp()
        if name == "particle_density":
            return sim._density
        if name == "sample_particle_index_short":
            return sim._sample_index
        if name in ("particle_Jp", "particle_external_force"):  # allocated, never written (:63-65)
            shape = (n,) if name == "particle_Jp" else (n, 3)
            return torch.zeros(shape, dtype=torch.float32, device=sim.device)
        if name == "particle_F_trial":
            raise AttributeError("particle_F_trial is not kept: F_trial lives only inside G2P, which "
                                 "stores the return-mapped F (particle_F)")
        if name in ("neighboring_cells", "neighboring_cells_grid_v"):
            return getattr(sim._reduced_grid(), name)
        if name in ("grid_m", "grid_v_in", "grid_v_out"):
            if sim._grid_from_reduced:  # the dense grid of the last p2g2p_reduced
                return getattr(sim._reduced_grid(), name)
            gm, gvin, gvout = eng.export_grid(0)
            return {"grid_m": gm, "grid_v_in": gvin, "grid_v_out": gvout}[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name == "sample_particle_index_short":
            self.__dict__["_sim"].load_sample_particle_index_from_tensor(value)
        else:
            super().__setattr__(name, value)


class MPMSimulator:
    """GB300 replacement of MPM_Simulator_WARP (engine_stress/mpm_solver_warp.py:24)."""

    def __init__(self, n_particles, n_grid=100, grid_lim=1.0, device="cuda:0", *,
                 chunk_size: int = 128):
        self._chunk_size = chunk_size
        self.initialize(n_particles, n_grid, grid_lim, device=device)

    # --------------------------------------------------------------- set-up
    def initialize(self, n_particles, n_grid=100, grid_lim=1.0, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:28-87 (defaults E=1000, nu=0.3, phi=25, g=0)."""
        self.n_particles = int(n_particles)
        mu, lam = lame_from_E_nu(1000.0, 0.3)
        self._params = SceneParams(n_particles=self.n_particles, n_grid=int(n_grid),
                                   grid_lim=float(grid_lim), material=A.JELLY, mu=mu, lam=lam,
                                   friction_angle=25.0, gravity=(0.0, 0.0, 0.0))
        self._E, self._nu = 1000.0, 0.3
        self._engine = MPMEngine([self._params], device=device, chunk_size=self._chunk_size)
        self.device = self._engine.device
        self._density = torch.zeros(self.n_particles, dtype=torch.float32, device=self.device)
        self._f_disp_loaded = None
        # sample_particle_index_short starts as one zero index (mpm_solver_warp.py:83)
        self._sample_index = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._reduced = None
        self._grid_from_reduced = False
        # colour for the OBJ output (mpm_solver_warp.py:71)
        self.particle_color = np.ones(self.n_particles, dtype=float)
        self.time = 0.0
        self.mpm_model = _Model(self)
        self.mpm_state = _State(self)

    @property
    def engine(self) -> MPMEngine:
        """The device engine (buffers and C-ABI driver) behind this simulator."""
        return self._engine

    def set_stress_surrogate(self, surrogate) -> None:
        """Take the sand return map + stress of each p2g2p from a trained
        ``surrogate.StressSurrogate`` (gated, SVD fallback); None restores
        the plain path."""
        self._engine.set_stress_surrogate(surrogate)

    @property
    def on_error(self) -> str:
        return self._engine.on_error

    @on_error.setter
    def on_error(self, v: str) -> None:
        if v not in ("raise", "warn", "ignore"):
            raise ValueError(v)
        self._engine.on_error = v

    def set_parameters(self, device="cuda:0", **kwargs):
        """engine_stress/mpm_solver_warp.py:89-127, plus E/nu/gravity/particle_vol."""
        p = self._params
        if "material" in kwargs:
            p.material = material_code(kwargs["material"])
        regrid = False
        if "grid_lim" in kwargs:
            p.grid_lim = float(kwargs["grid_lim"])
            regrid = True
        if "n_grid" in kwargs:
            p.n_grid = int(kwargs["n_grid"])
            regrid = True
        if "E" in kwargs or "nu" in kwargs:
            self._E = float(kwargs.get("E", self._E))
            self._nu = float(kwargs.get("nu", self._nu))
            p.mu, p.lam = lame_from_E_nu(self._E, self._nu)
        if "mu" in kwargs:
            p.mu = float(kwargs["mu"])
        if "lam" in kwargs:
            p.lam = float(kwargs["lam"])
        if "hardening" in kwargs:
            p.hardening = int(kwargs["hardening"])
        if "xi" in kwargs:
            p.xi = float(kwargs["xi"])
        if "friction_angle" in kwargs:
            p.friction_angle = float(kwargs["friction_angle"])
        if "g" in kwargs:
            p.gravity = (0.0, -float(kwargs["g"]), 0.0)  # mpm_utils.py:236
        if "gravity" in kwargs:
            g = tuple(float(x) for x in kwargs["gravity"])
            if len(g) != 3:
                raise ValueError("gravity must have 3 components")
            p.gravity = g
        self._engine.update_scenes(regrid=regrid)
        if "yield_stress" in kwargs:
            self._engine.load(A.FIELD_YIELD, torch.full((self.n_particles,),
                                                        float(kwargs["yield_stress"])))
        if "particle_vol" in kwargs:
            self.load_vol_from_tensor(torch.broadcast_to(
                torch.as_tensor(kwargs["particle_vol"], dtype=torch.float32),
                (self.n_particles,)))
        if "density" in kwargs:
            # set_value_to_float_array + get_float_array_product (:121-124)
            self._density = torch.full((self.n_particles,), float(kwargs["density"]),
                                       dtype=torch.float32, device=self.device)
            vol = self._engine.export(A.FIELD_VOL)
            self._engine.load(A.FIELD_MASS, self._density * vol)

    # --------------------------------------------------------------- loaders
    def load_x_initial_from_tensor(self, tensor_x_iniital, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:229-230"""
        self._engine.load(A.FIELD_X_INITIAL, tensor_x_iniital)

    def load_mass_from_tensor(self, tensor_mass, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:231-232"""
        self._engine.load(A.FIELD_MASS, tensor_mass)

    def load_uvF_from_tensor(self, tensor_u, tensor_v, tensor_F, clone=True, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:234-245.  Sets u, v and F_disp; as in the
        reference, the substep keeps reading particle_F, so F_disp only shows in
        exports until the next substep overwrites it with F - I."""
        self._engine.load(A.FIELD_U, tensor_u)
        self._engine.load(A.FIELD_V, tensor_v)
        self._f_disp_loaded = torch.as_tensor(tensor_F).detach().to(
            self.device, torch.float32).reshape(self.n_particles, 3, 3).clone()

    def load_C_from_tensor(self, tensor_C, clone=True, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:247-251"""
        self._engine.load(A.FIELD_C, tensor_C)

    def load_uvstress_from_tensor(self, tensor_u, tensor_v, tensor_stress, clone=True,
                                  device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:253-266 (the learned-stress hook)."""
        self._engine.load_uvstress(torch.as_tensor(tensor_u), torch.as_tensor(tensor_v),
                                   torch.as_tensor(tensor_stress))

    # extensions (no reference counterpart)
    def load_stress_from_decoder(self, decoder, label, mu=None):
        """The reduced-order loop's stress source: decode every particle's stress
        with a ``decoder.StressDecoder`` (NetDec, CROMnet_secondary.py:203-301) from
        the frame's label, the particle's x_initial and its mu row, straight into
        the state the next p2g2p reads (the reference decodes on the host side and
        calls load_uvstress_from_tensor, :253-266).  mu defaults to the friction
        angle of every particle, the parameter the reference's frames carry
        (:385-386)."""
        if mu is None and decoder.mu_dim == 1:
            mu = torch.full((self.n_particles, 1), float(self._params.friction_angle),
                            dtype=torch.float32, device=self.device)
        decoder.stress_into(self._engine, label, mu)

    def load_vol_from_tensor(self, tensor_vol):
        self._engine.load(A.FIELD_VOL, tensor_vol)

    def load_F_from_tensor(self, tensor_F):
        self._engine.load(A.FIELD_F, tensor_F)

    def load_yield_from_tensor(self, tensor_yield):
        self._engine.load(A.FIELD_YIELD, tensor_yield)

    def load_v_from_tensor(self, tensor_v):
        self._engine.load(A.FIELD_V, tensor_v)

    # --------------------------------------------------------------- substep
    def p2g2p(self, step, dt, print_norm=False, device="cuda:0"):
        """One substep, engine_stress/mpm_solver_warp.py:156-203."""
        self._engine.substep(float(self.time), float(dt))
        self._f_disp_loaded = None
        self._grid_from_reduced = False
        self.time = self.time + dt
        if print_norm:
            u, v, fd, st = self.export_uvFstress_from_warp()
            print("at mpm step", step, end=" ")
            print("norm of u, v, F_disp, stress, respectively: ",
                  "{:.4f}".format(float(torch.linalg.norm(u))),
                  "{:.4f}".format(float(torch.linalg.norm(v))),
                  "{:.4f}".format(float(torch.linalg.norm(fd))),
                  "{:.4f}".format(float(torch.linalg.norm(st))))

    def check_status(self) -> int:
        """Wait for the last substep's status word and act on it (``on_error``)."""
        return self._engine.poll_status(wait=True)

    # --------------------------------------------------------------- readers
    def _f_disp(self) -> torch.Tensor:
        if self._f_disp_loaded is not None:
            return self._f_disp_loaded.clone()
        return self._engine.export(A.FIELD_F_DISP).reshape(self.n_particles, 3, 3)

    def export_uvFstress_from_warp(self, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:305-310 -> (u, v, F_disp, stress)."""
        n = self.n_particles
        u, v, fd, st = self._engine.export_uvFstress()
        fd = self._f_disp_loaded.clone() if self._f_disp_loaded is not None else fd.reshape(n, 3, 3)
        return u.reshape(n, 3), v.reshape(n, 3), fd, st.reshape(n, 3, 3)

    # --------------------------------------------------------------- frame files
    def export_frame_arrays(self) -> dict:
        """The float32 arrays of one frame file in its transposed layout
        (mpm_export_frame, one device pass), as NumPy arrays."""
        n = self.n_particles
        buf = torch.empty(34 * n, dtype=torch.float32, device=self.device)
        eng = self._engine
        A.check(eng.lib.mpm_export_frame(ctypes.byref(eng.buf), buf.data_ptr(), eng.stream), "mpm_export_frame")
        arrays = FR.split_frame_buffer(buf.cpu().numpy(), n)
        if self._f_disp_loaded is not None:  # F_disp held apart from F (load_uvF, reduced substep)
            arrays["f_tensor"] = self._f_disp_loaded.reshape(n, 9).t().contiguous().cpu().numpy()
        return arrays

    def save_data_at_frame(self, dir_name, frame, include_parameter="friction_angle", save_to_h5=True,
                           save_to_obj=True, save_visual_F=False):
        """engine_stress/mpm_solver_warp.py:339-404: x, q, time, masses, f_tensor,
        stress (6 components), v, mu, C to dir_name/h5_f_<frame>.h5 (.npz without
        h5py), positions to the matching .obj.  The process umask is left alone
        (the reference sets it to 0) and the debug prints are dropped."""
        os.makedirs(dir_name, 0o777, exist_ok=True)
        fullfilename = FR.frame_filename(dir_name, frame)
        stem = fullfilename[: fullfilename.rindex(".")]
        if save_to_obj:
            self.particle_position2obj(stem + ".obj")
        if save_visual_F:
            self.particle_F_norm2obj(dir_name + "/visualF_f_" + str(frame).zfill(10) + ".obj")
        if not save_to_h5:
            return
        if include_parameter and include_parameter != "friction_angle":
            raise ValueError(f"include_parameter {include_parameter!r}: only 'friction_angle' is defined")
        a = self.export_frame_arrays()
        n = self.n_particles
        data = {"x": a["x"], "q": a["q"], "time": np.array([self.time]).reshape(1, 1), "masses": a["masses"],
                "f_tensor": a["f_tensor"], "stress": a["stress"], "v": a["v"]}
        if include_parameter:
            data["mu"] = np.ones((1, n)) * self._params.friction_angle
        data["C"] = a["C"]
        FR.write_frame(fullfilename, data)

    def particle_position2obj(self, fullfilename):
        """engine_stress/mpm_solver_warp.py:312-322: 'v x y z c c c' per particle,
        current positions, c = 1 - 1 / particle_color (all ones: 0.0)."""
        x = self._engine.export(A.FIELD_X).reshape(self.n_particles, 3).cpu().numpy()
        col = 1.0 - 1.0 / self.particle_color
        with open(fullfilename, "w") as f:
            f.write(FR.obj_lines(x, [(c, c, c) for c in col]))

    def particle_F_norm2obj(self, fullfilename, F_upperbound=2.0):
        """engine_stress/mpm_solver_warp.py:324-336: initial positions coloured by
        min(1, |F_disp| / F_upperbound)."""
        n = self.n_particles
        x0 = self._engine.export(A.FIELD_X_INITIAL).reshape(n, 3).cpu().numpy()
        fd = self._f_disp().reshape(n, 9).cpu().numpy()
        norm = np.linalg.norm(fd, axis=1)
        with open(fullfilename, "w") as f:
            f.write(FR.obj_lines(x0, [(np.minimum(1.0, c / F_upperbound), 0, 0) for c in norm]))

    def load_from_sampling(self, sampling_h5, n_grid=100, grid_lim=1.0, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:129-153: re-initialise for the file's
        particles; x_initial = x, v = 0, F_disp = f_tensor, F = I, mass, density,
        volume.  A missing file raises FileNotFoundError (the reference exits)."""
        d = FR.read_frame(FR.resolve(sampling_h5))
        x = np.asarray(d["x"]).transpose()
        q = np.asarray(d["q"]).transpose()
        n = q.shape[0]
        self.initialize(n, n_grid, grid_lim, device=device)
        mass = np.squeeze(np.asarray(d["masses"]), 0)
        density = np.squeeze(np.asarray(d["particle_density"]), 0)
        vol = np.squeeze(np.asarray(d["particle_volume"]), 0)
        self.load_x_initial_from_tensor(torch.from_numpy(np.ascontiguousarray(x, np.float32)))
        self.load_mass_from_tensor(torch.from_numpy(np.ascontiguousarray(mass, np.float32)))
        self.load_vol_from_tensor(torch.from_numpy(np.ascontiguousarray(vol, np.float32)))
        self._density = torch.from_numpy(np.ascontiguousarray(density, np.float32)).to(self.device)
        f = np.ascontiguousarray(np.asarray(d["f_tensor"], np.float32).reshape(n, 3, 3))
        self._f_disp_loaded = torch.from_numpy(f).to(self.device)

    def load_uvFstress_from_h5(self, h5filename, sample_point=0, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:268-303: u = q, v, stress from its six
        components; f_tensor is read but, as there, not loaded."""
        d = FR.read_frame(FR.resolve(h5filename))
        q = np.asarray(d["q"]).transpose()
        v = np.asarray(d["v"]).transpose()
        stress = FR.stress_from_components(np.asarray(d["stress"]).transpose())
        self.load_uvstress_from_tensor(torch.from_numpy(np.ascontiguousarray(q, np.float32)),
                                       torch.from_numpy(np.ascontiguousarray(v, np.float32)),
                                       torch.from_numpy(np.ascontiguousarray(stress, np.float32)))

    # --------------------------------------------------------------- colliders
    def add_surface_collider(self, point, normal, surface="sticky", friction=0.0,
                             start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:407-451"""
        self._params.colliders.append(Collider.surface(point, normal, surface, friction,
                                                       start_time, end_time))
        self._engine.update_scenes()

    def add_bounding_box(self, start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:499-525"""
        self._params.colliders.append(Collider.bounding_box(start_time, end_time))
        self._engine.update_scenes()

    def _add_collider(self, c: Collider) -> None:
        self._params.colliders.append(c)
        self._engine.update_scenes()

    # add_surface_collider2 (mpm_solver_warp.py:453-497) writes zero for every
    # surface type too (:495): the same collider
    add_surface_collider2 = add_surface_collider

    def set_velocity_on_infinite_plane(self, point, normal, velocity, threshold, start_time=0.0, end_time=999.0,
                                       reset=0):
        """engine_stress/mpm_solver_warp.py:527-568"""
        self._add_collider(Collider.velocity_plane(point, normal, velocity, threshold, start_time, end_time, reset))

    def set_column_moving_as_circle(self, R, radius, height, v_scale, start_time=0.0, end_time=999.0):
        """engine_stress/mpm_solver_warp.py:570-607"""
        self._add_collider(Collider.circle_column(R, radius, height, v_scale, start_time, end_time))

    def set_rotation_on_disk(self, point, normal, radius, width, v_scale, start_time=0.0, end_time=999.0, reset=0):
        """engine_stress/mpm_solver_warp.py:609-665"""
        self._add_collider(Collider.rotating_disk(point, normal, radius, width, v_scale, start_time, end_time,
                                                  reset))

    def set_velocity_on_cube(self, point, width, velocity, start_time=0.0, end_time=999.0, reset=0):
        """engine_stress/mpm_solver_warp.py:667-695"""
        self._add_collider(Collider.velocity_cube(point, width, velocity, start_time, end_time, reset))

    def add_sphere_leader(self, center, radius, velocity, start_time=0, end_time=999):
        """engine_stress/mpm_solver_warp.py:697-720"""
        self._add_collider(Collider.sphere(center, radius, velocity, start_time, end_time))

    # --------------------------------------------------------------- reduced substep
    def load_sample_particle_index_from_tensor(self, tensor_index):
        """Extension: the sample list (sample_particle_index_short, warp_utils.py:120),
        user particle indices."""
        t = torch.as_tensor(tensor_index).detach().reshape(-1)
        if t.dtype.is_floating_point or t.dtype == torch.bool:
            raise TypeError("sample indices must be integers")
        self._sample_index = t.to(device=self.device, dtype=torch.int32).contiguous()

    def _reduced_grid(self) -> ReducedGrid:
        ng = self._params.n_grid
        if self._reduced is None or self._reduced.n_grid != ng:
            self._reduced = ReducedGrid(ng, self.device)
        rg = self._reduced
        rg.sample_index = self._sample_index
        rg.density = self._density.contiguous()
        return rg

    def _f_disp_state(self) -> torch.Tensor:
        """particle_F_disp as its own array: F - I after a substep, the loaded
        tensor after load_uvF_from_tensor; the reduced kernels read and write it."""
        if self._f_disp_loaded is None:
            self._f_disp_loaded = self._engine.export(A.FIELD_F_DISP).reshape(self.n_particles, 3, 3)
        return self._f_disp_loaded

    def p2g2p_reduced(self, step, dt, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:214-227: the grid of the sample points'
        neighbourhood (mpm_state.grid_m / grid_v_in / grid_v_out); particles whose
        base cell is marked set F = F_disp + I; nothing moves; time += dt."""
        rg = self._reduced_grid()
        rg.f_disp = self._f_disp_state()
        self._engine.p2g2p_reduced(rg, float(self.time), float(dt))
        self._grid_from_reduced = True
        self.time = self.time + dt

    def experiment_for_C(self, device="cuda:0"):
        """engine_stress/mpm_solver_warp.py:207-209: adds the -2..4 marks of the
        sample points and returns neighboring_cells_grid_v (the live array)."""
        rg = self._reduced_grid()
        rg.f_disp = self._f_disp_state()
        self._engine.mark_neighboring_cells_grid_v(rg)
        return rg.neighboring_cells_grid_v

    def g2p_sample(self, dt, device="cuda:0"):
        """Extension: launch g2p_sample (engine_stress/mpm_utils.py:415-471) on the
        grid of the last p2g2p_reduced.  The sample particles take v, x, F and
        F_disp from grid_v_out; yield_stress is read at the sample's list
        position, as there (:464)."""
        rg = self._reduced_grid()
        rg.f_disp = self._f_disp_state()
        self._engine.g2p_sample(rg, float(dt))


MPM_Simulator_WARP = MPMSimulator

__all__ = ["MPMSimulator", "MPM_Simulator_WARP", "MPMStatusError", "flatten2nD"]
