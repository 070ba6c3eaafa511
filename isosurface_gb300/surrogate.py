"""The learned SDF surrogate: a Fourier-feature MLP trained on the GPU by the
library's own kernels (csrc/mlp.cu), evaluated with BF16 tensor cores
(csrc/mlp_infer.cu), and used to mesh an expensive source with exact
re-sampling near the surface."""
import ctypes
import os

import numpy as np

from ._capi import (ISO_FLAG_KEYS, ISO_SURROGATE_EXACT_COARSE, ISO_SURROGATE_WITNESS, MeshDistance, MeshInfo,
                    SurrogateStats, check, lib)

f32p = ctypes.POINTER(ctypes.c_float)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


class Surrogate:
    def __init__(self, ctx, seed=1):
        self.ctx = ctx
        h = ctypes.c_void_p()
        check(lib().iso_mlp_create(ctx.h, seed, ctypes.byref(h)), ctx.h)
        self.h = h
        self.nparams = int(lib().iso_mlp_num_params())

    def close(self):
        if getattr(self, "h", None):
            lib().iso_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        p = np.empty(self.nparams, np.float32)
        check(lib().iso_mlp_get_params(self.h, p.ctypes.data_as(f32p)), self.ctx.h)
        return p

    @params.setter
    def params(self, p):
        p = _f32(p)
        assert p.size == self.nparams
        check(lib().iso_mlp_set_params(self.h, p.ctypes.data_as(f32p)), self.ctx.h)

    def forward(self, points, bf16=False):
        """Network values at host points: the fp32 SIMT path, or with bf16=True
        the tcgen05 tensor-core path (bf16 operands, fp32 accumulation)."""
        pts = _f32(points).reshape(-1, 3)
        out = np.empty(len(pts), np.float32)
        fn = lib().iso_mlp_forward_bf16 if bf16 else lib().iso_mlp_forward
        check(fn(self.h, pts.ctypes.data_as(f32p), len(pts), out.ctypes.data_as(f32p)), self.ctx.h)
        return out

    def loss_grad(self, points, targets, clamp_d=0.1):
        pts = _f32(points).reshape(-1, 3)
        t = _f32(targets)
        loss = ctypes.c_float()
        g = np.empty(self.nparams, np.float32)
        check(lib().iso_mlp_loss_grad(self.h, pts.ctypes.data_as(f32p), t.ctypes.data_as(f32p), len(pts), clamp_d,
                                      ctypes.byref(loss), g.ctypes.data_as(f32p)), self.ctx.h)
        return loss.value, g

    def make_dataset(self, exact_source, n, lo=-1.0, hi=1.0, seed=5):
        prog = self.ctx.program(exact_source)
        check(lib().iso_mlp_make_dataset(self.h, prog.h, n, lo, hi, seed), self.ctx.h)

    def train(self, steps, batch=65536, lr=1e-3, clamp_d=0.1, seed=11):
        hist = np.empty(steps, np.float32)
        check(lib().iso_mlp_train(self.h, steps, batch, lr, clamp_d, seed, hist.ctypes.data_as(f32p)), self.ctx.h)
        return hist

    def save(self, path):
        """Checkpoint of the training state: parameters, Adam moments and step."""
        check(lib().iso_mlp_save(self.h, os.fsencode(path)), self.ctx.h)

    def load(self, path):
        """Restore a checkpoint written by save (the dataset stays as it is)."""
        check(lib().iso_mlp_load(self.h, os.fsencode(path)), self.ctx.h)

    def field(self, exact_source, size, field_ptr, pitch, coarse_step=4, band_cells=2.0):
        """The surrogate field of MarchingCubes::new(size) into a device buffer
        laid out as Context.sample_grid writes it; returns the band statistics."""
        st = SurrogateStats()
        check(lib().iso_surrogate_field(self.ctx.h, self.h, self.ctx.program(exact_source).h, size, coarse_step,
                                        band_cells, ctypes.c_void_p(field_ptr), pitch, ctypes.byref(st)),
              self.ctx.h)
        return _stats(st)

    def field_ex(self, exact_source, size, field_ptr, pitch, coarse_step=4, band_cells=2.0, exact_coarse=False,
                 witness=False):
        """iso_surrogate_field_ex: exact_coarse builds the coarse grid from the
        exact source instead of the network (the pipeline without the
        network); witness adds the spot checks at the sphere-set source's
        witness points.  Returns the band statistics with the number of
        flagged spheres."""
        st, flagged = SurrogateStats(), ctypes.c_uint64()
        flags = (ISO_SURROGATE_EXACT_COARSE if exact_coarse else 0) | (ISO_SURROGATE_WITNESS if witness else 0)
        check(lib().iso_surrogate_field_ex(self.ctx.h, None if exact_coarse else self.h,
                                           self.ctx.program(exact_source).h, size, coarse_step, band_cells, flags,
                                           ctypes.c_void_p(field_ptr), pitch, ctypes.byref(st), ctypes.byref(flagged)),
              self.ctx.h)
        out = _stats(st)
        out["flagged"] = int(flagged.value)
        return out

    def extract(self, exact_source, size, coarse_step=4, band_cells=2.0, keys=False):
        """Marching cubes over the surrogate field; the mesh stays in the
        context (Context.download).  Returns (MeshInfo, band statistics)."""
        st, info = SurrogateStats(), MeshInfo()
        self.ctx._vertex_floats = 3
        check(lib().iso_surrogate_extract(self.ctx.h, self.h, self.ctx.program(exact_source).h, size, coarse_step,
                                          band_cells, ISO_FLAG_KEYS if keys else 0, ctypes.byref(st),
                                          ctypes.byref(info)), self.ctx.h)
        return info, _stats(st)


def _stats(st):
    return {"coarse_points": st.coarse_points, "band_points": st.band_points, "total_points": st.total_points}


def checkpoint_info(path):
    """(parameter count, Adam steps) of a checkpoint; needs no device."""
    n, step = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().iso_mlp_checkpoint_info(os.fsencode(path), ctypes.byref(n), ctypes.byref(step)))
    return n.value, step.value


def mesh_distance(ctx, a, b, bucket, max_rings=32):
    """Nearest-vertex distances between vertex arrays a and b (n x >=3, the
    first three columns are xyz): Chamfer (mean of the two directed means),
    Hausdorff (larger directed max), both directed figures and the number of
    vertices whose search stopped at max_rings."""
    a = _f32(np.asarray(a)[:, :3])
    b = _f32(np.asarray(b)[:, :3])
    r = MeshDistance()
    check(lib().iso_mesh_distance(ctx.h, a.ctypes.data_as(f32p), len(a), b.ctypes.data_as(f32p), len(b), bucket,
                                  max_rings, ctypes.byref(r)), ctx.h)
    return {"chamfer": 0.5 * (r.mean_ab + r.mean_ba), "hausdorff": max(r.max_ab, r.max_ba), "mean_ab": r.mean_ab,
            "mean_ba": r.mean_ba, "max_ab": r.max_ab, "max_ba": r.max_ba, "capped": int(r.capped)}


def case_disagreement(ctx, field_a, field_b, nx, ny, nz, pitch):
    """Cells whose corner signs differ between two device fields."""
    n = ctypes.c_uint64()
    check(lib().iso_field_case_disagreement(ctx.h, ctypes.c_void_p(field_a), ctypes.c_void_p(field_b), nx, ny, nz,
                                            pitch, ctypes.byref(n)), ctx.h)
    return int(n.value)
