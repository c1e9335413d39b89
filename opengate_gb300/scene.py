"""Host-side scene: the numpy arrays and ctypes descriptors of one simulation.

A :class:`Scene` owns every host buffer that the C ABI reads (tables, label
image, majorant, source spectra) and builds the descriptor structs pointing at
them, so the same scene can be handed to the GPU engine or, in the tests, to
the CPU oracle.
"""

import math

import numpy as np

from . import _capi as C
from . import tables as T


class SourceSpec:
    """Primary generator parameters (GenericSource subset), SI-free: mm, rad, MeV."""

    def __init__(self):
        self.pos_type = C.GG_POS_POINT
        self.translation = [0.0, 0.0, 0.0]
        self.rotation = np.eye(3)
        self.half_size = [0.0, 0.0, 0.0]
        self.radius = 0.0
        self.dir_type = C.GG_DIR_ISO
        self.theta = [0.0, math.pi]
        self.phi = [0.0, 2.0 * math.pi]
        self.momentum = [0.0, 0.0, 1.0]
        self.focus = [0.0, 0.0, 0.0]
        self.accept_boxes = []  # list of (min xyz, max xyz)
        self.ff_angle_tolerance = 0.0  # angle check applied by a free flight (rad, 0 = none)
        # GG_DIR_FORCED (ForceDirection toward the SPECT heads): cone angles (rad)
        self.fd_angle_min = 0.0
        self.fd_angle_max = 0.0
        self.max_rejection = 10000
        self.ene_type = C.GG_ENE_MONO
        self.mono = 1.0
        self.spec_e = None
        self.spec_cdf = None
        self.e_lo = 0.0
        self.e_hi = 0.0
        # VoxelSource (pos_type GG_POS_VOXELS): activity grid and its CDFs
        self.vox_dims = [0, 0, 0]
        self.vox_spacing = [1.0, 1.0, 1.0]
        self.vox_corner = [0.0, 0.0, 0.0]
        self.cdf_z = self.cdf_y = self.cdf_x = None

    def set_activity_image(self, activity, spacing, corner):
        """VoxelSource placement: activity [z][y][x], spacing and outer corner (mm, world)."""
        from .spect import voxel_cdfs

        act = np.asarray(activity)
        self.pos_type = C.GG_POS_VOXELS
        self.vox_dims = [int(act.shape[2]), int(act.shape[1]), int(act.shape[0])]
        self.vox_spacing = [float(v) for v in spacing]
        self.vox_corner = [float(v) for v in corner]
        self.cdf_z, self.cdf_y, self.cdf_x = voxel_cdfs(act)

    def energy_bounds(self):
        if self.ene_type == C.GG_ENE_MONO:
            return self.mono, self.mono
        if self.ene_type == C.GG_ENE_RANGE:
            return self.e_lo, self.e_hi
        return float(np.min(self.spec_e)), float(np.max(self.spec_e))


class Scene:
    """Tables + image volume + world + source for one transport run."""

    def __init__(self, phys_tables, labels, spacing, corner, world_half, world_material, source):
        self.pt = phys_tables
        self.labels = np.ascontiguousarray(labels, dtype=np.uint16)  # [nz][ny][nx]
        if self.labels.ndim != 3:
            raise ValueError("labels must be a 3D array [nz][ny][nx]")
        if int(self.labels.max(initial=0)) >= len(phys_tables.materials):
            raise ValueError("label image refers to a material index outside the table")
        self.spacing = [float(v) for v in spacing]
        self.corner = [float(v) for v in corner]
        self.world_half = [float(v) for v in world_half]
        self.world_material = int(world_material)
        self.source = source
        present = np.unique(self.labels)
        self.majorant = np.ascontiguousarray(phys_tables.majorant(present), dtype=np.float32)
        lo, hi = source.energy_bounds()
        if lo < T.E_MIN or hi > T.E_MAX:
            raise ValueError(f"source energies [{lo}, {hi}] MeV outside the tables [{T.E_MIN}, {T.E_MAX}]")
        self._build_descs()

    def tle_desc(self, threshold_energy=float("inf"), energy_min=0.0, database="EPDL"):
        """Descriptor of the track-length estimator (gg_set_tle) for these tables;
        the mu_en table is kept alive by the scene."""
        self._muen = np.ascontiguousarray(self.pt.muen(database), dtype=np.float32)
        return C.TleDesc(1, float(threshold_energy), float(energy_min), C.ptr(self._muen, C.ctypes.c_float))

    @property
    def dims_xyz(self):
        nz, ny, nx = self.labels.shape
        return nx, ny, nz

    def _build_descs(self):
        pt = self.pt
        self._sig = np.ascontiguousarray(pt.sig, dtype=np.float32)
        self._cum = np.ascontiguousarray(pt.cum, dtype=np.float32)
        self._ray_amax = np.ascontiguousarray(pt.ray_amax, dtype=np.float32)
        self._ray_cum = np.ascontiguousarray(pt.ray_cum, dtype=np.float32)
        self._mat_comp = np.ascontiguousarray(pt.mat_comp, dtype=np.int32)
        self._mat_rho = np.ascontiguousarray(pt.mat_rho, dtype=np.float32)
        t = C.TablesDesc()
        t.n_e = T.N_E
        t.ln_emin = float(np.float32(math.log(T.E_MIN)))
        t.inv_dln = float(np.float32((T.N_E - 1) / (math.log(T.E_MAX) - math.log(T.E_MIN))))
        t.e_min = float(np.float32(T.E_MIN))
        t.e_max = float(np.float32(T.E_MAX))
        t.n_comp = pt.n_comp
        t.sig = C.ptr(self._sig, C.ctypes.c_float)
        t.cum = C.ptr(self._cum, C.ctypes.c_float)
        t.ray_amax = C.ptr(self._ray_amax, C.ctypes.c_float)
        t.n_ray = T.N_RAY
        self._ray_x2 = np.ascontiguousarray(T.rayleigh_x2_nodes(), dtype=np.float32)
        t.ray_x2 = C.ptr(self._ray_x2, C.ctypes.c_float)
        t.ray_cum = C.ptr(self._ray_cum, C.ctypes.c_float)
        t.n_mat = len(pt.materials)
        t.mat_comp = C.ptr(self._mat_comp, C.ctypes.c_int32)
        t.mat_rho = C.ptr(self._mat_rho, C.ctypes.c_float)
        self.tables_desc = t

        v = C.VolumeDesc()
        nx, ny, nz = self.dims_xyz
        v.dims[:] = [nx, ny, nz]
        v.spacing[:] = self.spacing
        v.corner[:] = self.corner
        v.labels = C.ptr(self.labels, C.ctypes.c_uint16)
        v.majorant = C.ptr(self.majorant, C.ctypes.c_float)
        self.volume_desc = v

        w = C.WorldDesc()
        w.half_size[:] = self.world_half
        w.material = self.world_material
        self.world_desc = w

        s = self.source
        d = C.SourceDesc()
        d.pos_type = s.pos_type
        d.translation[:] = [float(x) for x in s.translation]
        d.rotation[:] = [float(x) for x in np.asarray(s.rotation, dtype=np.float64).ravel()]
        d.half_size[:] = [float(x) for x in s.half_size]
        d.radius = float(s.radius)
        d.dir_type = s.dir_type
        d.theta[:] = [float(x) for x in s.theta]
        d.phi[:] = [float(x) for x in s.phi]
        d.momentum[:] = [float(x) for x in s.momentum]
        d.focus[:] = [float(x) for x in s.focus]
        self._acc = np.ascontiguousarray(
            np.array([list(lo) + list(hi) for lo, hi in s.accept_boxes], dtype=np.float64).reshape(-1)
        ) if s.accept_boxes else np.zeros(6, dtype=np.float64)
        d.n_accept = len(s.accept_boxes)
        d.accept_boxes = C.ptr(self._acc, C.ctypes.c_double)
        d.max_rejection = int(s.max_rejection)
        d.ene_type = s.ene_type
        d.mono = float(s.mono)
        self._spec_e = np.ascontiguousarray(s.spec_e if s.spec_e is not None else np.zeros(2), dtype=np.float64)
        self._spec_cdf = np.ascontiguousarray(s.spec_cdf if s.spec_cdf is not None else np.ones(1), dtype=np.float64)
        d.n_spec = int(len(s.spec_cdf)) if s.spec_cdf is not None else 0
        d.spec_e = C.ptr(self._spec_e, C.ctypes.c_double)
        d.spec_cdf = C.ptr(self._spec_cdf, C.ctypes.c_double)
        d.e_lo = float(s.e_lo)
        d.e_hi = float(s.e_hi)
        d.vox_dims[:] = s.vox_dims
        d.vox_spacing[:] = s.vox_spacing
        d.vox_corner[:] = s.vox_corner
        self._cdfs = [np.ascontiguousarray(c if c is not None else np.ones(1), dtype=np.float32)
                      for c in (s.cdf_z, s.cdf_y, s.cdf_x)]
        d.cdf_z, d.cdf_y, d.cdf_x = (C.ptr(c, C.ctypes.c_float) for c in self._cdfs)
        d.fd_cos_min = math.cos(float(s.fd_angle_min))
        d.fd_cos_max = math.cos(float(s.fd_angle_max))
        self.source_desc = d

    def set_source(self, source):
        """Replaces the source (validated like the constructor) and rebuilds the descriptors."""
        lo, hi = source.energy_bounds()
        if lo < T.E_MIN or hi > T.E_MAX:
            raise ValueError(f"source energies [{lo}, {hi}] MeV outside the tables [{T.E_MIN}, {T.E_MAX}]")
        self.source = source
        self._build_descs()

    def source_desc_bytes(self):
        """Bytes of the source arrays a gg_set_source call copies to the device."""
        return int(self._acc.nbytes + self._spec_e.nbytes + self._spec_cdf.nbytes + sum(c.nbytes for c in self._cdfs))

    @property
    def n_voxels(self):
        return int(self.labels.size)

    def voxel_density(self):
        """g/cm3 per voxel, float64, shape of the label image."""
        return self.pt.mat_rho.astype(np.float64)[self.labels]
