"""
Neighbour-consistent sign adjustment of the vesselness main directions and
their completion to full frames -- the drop-in for the reference module of the
same name (src/processing/adjust_directions.py).

AdvancedAdjuster keeps the reference's sequence (adjust_directions.py:213-256):
ridge candidates on the GPU, hysteresis on the host, main directions on the
GPU, the minimum spanning tree over the ridge points (ridge_mst.py: the tree
of SciPy's Kruskal with a stable order of equal distances, without the
reference's dense R x R matrix; its local phase in Boruvka rounds on the
GPU), the sign propagation along it on the host, ridge
cleaning on the host, and the nearest-ridge sign flip of every voxel on the
GPU (m16_adjust_nonridge_signs_indexed: the reference's brute-force nearest
ridge point, found through a cell index of the ridge points).  TransformationCompleter
runs m16_complete_transformations.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _native as N
from .labeling import label26, label_device
from .parameters import TreePrintable
from .ridge_detection import RawRidgeDetector, hysteresis_threshold
from .ridge_mst import propagate_signs, propagate_signs_device, ridge_mst_edges


class AdvancedAdjuster(TreePrintable):
    """adjust_directions.py:25-446"""

    # where the local phase of the ridge MST runs: "gpu" (m16_ridge_mst_local)
    # or "host" (the same edges with SciPy's Kruskal)
    mst_local = "gpu"
    # where the 26-connected labelling of the hysteresis and the cleaning
    # runs: "gpu" (m16_label26) or "host" (scipy.ndimage.label, the same labels)
    labeler = "gpu"

    def __init__(self, threshold, qeigs, response, voxel_size=1, ridge_detection_only=False, clean_ridge=True,
                 loader=None):
        self.__threshold = None
        self.__qeigs = None
        self.__response = None
        self.__voxel_size = None
        self.__ridge_detection_only = None
        self.__clean_ridge = None
        self.__ridge = None
        self.__main_dirs_unadjusted = None
        self._ridge_detector = None
        self._hysteresis = None
        self._dtype = np.float32
        self._loader = loader  # accepted for compatibility, unused
        if threshold is not None:
            self.threshold = threshold
        if qeigs is not None:
            self.qeigs = qeigs
        if response is not None:
            self.response = response
        if voxel_size is not None:
            self.voxel_size = voxel_size
        self.ridge_detection_only = ridge_detection_only
        self.clean_ridge = clean_ridge

    # -- properties (adjust_directions.py:105-186) -----------------------------
    @property
    def threshold(self):
        return self.__threshold

    @threshold.setter
    def threshold(self, value):
        try:
            len(value)
            value = tuple(sorted(value))
            self._hysteresis = True
            lower = value[0]
        except TypeError:
            self._hysteresis = False
            lower = value
        if value != self.__threshold:
            self.__threshold = value
            self._ridge_detector = RawRidgeDetector(self._loader, lower)

    @property
    def qeigs(self):
        return self.__qeigs

    @qeigs.setter
    def qeigs(self, value):
        self.__qeigs = np.require(value, dtype=self._dtype, requirements=["C", "A"])

    @property
    def response(self):
        return self.__response

    @response.setter
    def response(self, value):
        self.__response = np.require(value, dtype=self._dtype, requirements=["C", "A"])

    @property
    def voxel_size(self):
        return self.__voxel_size

    @voxel_size.setter
    def voxel_size(self, value):
        self.__voxel_size = tuple(np.multiply(np.ones(3), value))

    @property
    def ridge_detection_only(self):
        return self.__ridge_detection_only

    @ridge_detection_only.setter
    def ridge_detection_only(self, value):
        self.__ridge_detection_only = value

    @property
    def clean_ridge(self):
        return self.__clean_ridge

    @clean_ridge.setter
    def clean_ridge(self, value):
        self.__clean_ridge = value

    @property
    def ridge(self):
        """After execute(): the detected (and possibly cleaned) ridge."""
        return self.__ridge

    @property
    def main_dirs_unadjusted(self):
        """After execute(): the extracted, not yet adjusted main directions."""
        if self.__main_dirs_unadjusted is None and getattr(self, "_d_main_unadjusted", None) is not None:
            self.__main_dirs_unadjusted = self._d_main_unadjusted.cpu().numpy()
            self._d_main_unadjusted = None
        return self.__main_dirs_unadjusted

    # -- the sequence (adjust_directions.py:213-256) ---------------------------
    def execute(self, verbose=True):
        """Returns the sign-adjusted main directions, (z, y, x, 3) float32, or
        None when ridge_detection_only."""
        assert self.response.shape == self.qeigs.shape[:3] and self.qeigs.shape[3] == 3
        torch = N.torch_mod()
        self.timings = {}   # seconds per step of the last execute()
        self._d_qeigs = N.to_device_f32(self.qeigs)
        if self.labeler == "gpu" and self.mst_local == "gpu":
            adjusted = self._execute_device()
        else:
            adjusted = self._execute_host()
        del self._d_qeigs
        self._d_main = None
        torch.cuda.current_stream().synchronize()
        return adjusted

    def _execute_host(self):
        """The sequence with the volumes on the host (labeler or mst_local
        "host"): each step as the reference writes it."""
        with self._timed("ridge_candidates_and_hysteresis"):
            labeled_ridge = self._label_ridge()
        adjusted = None
        if (not self.ridge_detection_only) or self.clean_ridge:
            with self._timed("main_directions"):
                main_dirs = self._qeigs_to_main_dirs()
            # before cleaning, only the per-segment norms matter (see _adjust_ridge_directions)
            ridge_coords, ridge_dirs = self._adjust_ridge_directions(labeled_ridge, main_dirs,
                                                                     join_components=not self.clean_ridge)
            if self.clean_ridge:
                labeled_ridge = self._do_clean_ridge(labeled_ridge, ridge_coords, ridge_dirs)
                if not self.ridge_detection_only:
                    ridge_coords, ridge_dirs = self._adjust_ridge_directions(labeled_ridge, main_dirs)
            if not self.ridge_detection_only:
                with self._timed("nearest_ridge_flip"):
                    adjusted = self._adjust_all_directions(ridge_coords, ridge_dirs)
                self.ridge_coords, self.ridge_dirs = ridge_coords, ridge_dirs
        return adjusted

    def _execute_device(self):
        """The same sequence with every volume kept on the device: ridge
        candidates, hysteresis, the main directions, the labels of the
        cleaning and the cleaned ridge stay there, and only lists of ridge
        points (coordinates, their directions and labels) come to the host
        for the tree steps.  Gives _execute_host's bits."""
        self.__main_dirs_unadjusted = None
        self._d_main_unadjusted = None
        with self._timed("ridge_candidates_and_hysteresis"):
            d_ridge = self._label_ridge_dev()
        adjusted = None
        if (not self.ridge_detection_only) or self.clean_ridge:
            with self._timed("main_directions"):
                d_main = self._d_main
                self._d_main_unadjusted = d_main
                self._d_qeigs.copy_(d_main)
                self._d_main = None
            pts = self._ridge_points_dev(d_ridge)
            ridge_coords, ridge_dirs = self._adjust_ridge_directions_dev(pts, d_main,
                                                                         join_components=not self.clean_ridge)
            if self.clean_ridge:
                d_ridge = self._do_clean_ridge_dev(d_ridge, pts, ridge_dirs)
                if not self.ridge_detection_only:
                    pts = self._ridge_points_dev(d_ridge)
                    ridge_coords, ridge_dirs = self._adjust_ridge_directions_dev(pts, d_main)
            if not self.ridge_detection_only:
                with self._timed("nearest_ridge_flip"):
                    adjusted = self._adjust_all_directions(ridge_coords, ridge_dirs)
                self.ridge_coords, self.ridge_dirs = ridge_coords, ridge_dirs
        with self._timed("ridge_to_host"):
            self.__ridge = d_ridge.to(N.torch_mod().float32).cpu().numpy()
        return adjusted

    def _label_ridge_dev(self):
        """Ridge candidates and main directions in one pass
        (m16_detect_ridges_main_directions), then the hysteresis (m16_hysteresis)
        on the device.  Returns the ridge as a uint8 device mask; the main
        directions stay in self._d_main."""
        torch = N.torch_mod()
        L = N.lib()
        shape = tuple(int(v) for v in self.response.shape)
        resp = N.to_device_f32(self.response, shape)
        d_ridge = torch.empty(shape, dtype=torch.float32, device=N.device())
        self._d_main = torch.empty_like(self._d_qeigs)
        st = L.m16_detect_ridges_main_directions(N.ptr(resp), N.ptr(self._d_qeigs), shape[0], shape[1], shape[2],
                                                 float(self._ridge_detector.threshold), N.ptr(d_ridge),
                                                 N.ptr(self._d_main), N.stream_ptr())
        N.check("m16_detect_ridges_main_directions", st)
        cand = (d_ridge != 0).to(torch.uint8)
        if not self._hysteresis:
            return cand
        # sure = ridge & (response >= upper), compared in float32 as numpy does
        sure = (cand.bool() & (resp >= self.threshold[1])).to(torch.uint8)
        out = torch.empty(shape, dtype=torch.uint8, device=N.device())
        ws = N.workspace(L.m16_hysteresis_workspace_bytes(*shape))
        N.check("m16_hysteresis", L.m16_hysteresis(N.ptr(cand), N.ptr(sure), shape[0], shape[1], shape[2], N.ptr(out),
                                                   N.ptr(ws), ws.numel(), N.stream_ptr()))
        return out

    def _ridge_points_dev(self, d_mask):
        """(host int64 R x 3, device int64 R x 3) coordinates of the mask's
        voxels in C order (np.argwhere's order)."""
        with self._timed("ridge_coordinates"):
            d_coords = N.torch_mod().nonzero(d_mask)
            return d_coords.cpu().numpy(), d_coords

    def _adjust_ridge_directions_dev(self, pts, d_main, join_components=True):
        """_adjust_ridge_directions on the device mask: the directions are
        gathered at the ridge points on the device."""
        coords, d_coords = pts
        if len(coords) == 0:
            raise ValueError("no ridge points: nothing to propagate directions along")
        with self._timed("mst_local" if not join_components else "mst_local_and_joins"):
            shape = tuple(int(v) for v in self.response.shape)
            a, b = ridge_mst_edges(coords, self.voxel_size, join_components=join_components, local=self.mst_local,
                                   on_device=True, d_points=d_coords, box=((0, 0, 0), shape))
        with self._timed("sign_propagation"):
            d_dirs = d_main[d_coords[:, 0], d_coords[:, 1], d_coords[:, 2]]
            adjusted = propagate_signs_device(d_dirs, a, b).cpu().numpy()
        return np.asarray(coords, dtype=np.uint16, order="C"), adjusted

    def _do_clean_ridge_dev(self, d_mask, pts, ridge_dirs):
        """_do_clean_ridge on the device mask: labels on the device, the
        per-segment sums from the labels at the ridge points, the kept
        segments selected on the device.  Returns the cleaned uint8 mask."""
        torch = N.torch_mod()
        coords, d_coords = pts
        with self._timed("clean_labels"):
            d_comp, n_lab = label_device(d_mask, 26)
            point_label = d_comp[d_coords[:, 0], d_coords[:, 1], d_coords[:, 2]].cpu().numpy()
        with self._timed("clean_segment_sums"):
            sums = self._segment_sums(point_label, n_lab, ridge_dirs)
            kept = self._kept_segments(n_lab, len(coords) < d_mask.numel(), sums)
        keep = np.zeros(n_lab + 1, dtype=np.uint8)
        keep[np.asarray(kept, dtype=np.int64)] = 1
        return torch.from_numpy(keep).to(N.device())[d_comp.long()]

    def _segment_sums(self, point_label, n_lab, ridge_dirs):
        """(n_lab + 1) x 3 float64: per label the directions of its ridge
        points times the voxel size, summed in the C order of its voxels, one
        after the other (np.sum over axis 0 of the reference's list; np.bincount
        adds sequentially too).  The library's m16_segment_direction_sums does
        it in one pass where the reference's product is a double one (float32
        directions, a voxel size that numpy multiplies in double); otherwise
        np.bincount."""
        dirs = np.asarray(ridge_dirs)
        vs = np.asarray(self.__voxel_size)
        if (dirs.dtype == np.float32 and dirs.ndim == 2 and dirs.shape[1] == 3 and vs.dtype.kind in "iuf"
                and np.result_type(dirs.dtype, vs.dtype) == np.float64):
            dirs = np.ascontiguousarray(dirs)
            pl = np.ascontiguousarray(point_label, dtype=np.int32)
            v3 = np.ascontiguousarray(np.broadcast_to(vs.astype(np.float64), (3,)))
            sums = np.empty((n_lab + 1, 3), np.float64)
            vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
            N.check("m16_segment_direction_sums",
                    N.lib().m16_segment_direction_sums(vp(pl), vp(dirs), len(pl), vp(v3), n_lab + 1, vp(sums)))
            return sums
        scaled = dirs * self.__voxel_size   # float32 * tuple -> float64, as in the reference
        return np.stack([np.bincount(point_label, weights=scaled[:, k], minlength=n_lab + 1) for k in range(3)], -1)

    def _kept_segments(self, n_lab, has_background, sums):
        """The labels the cleaning keeps (adjust_directions.py:319-337): the
        ceil(3 ln(e + n)) segments with the longest summed (scaled) direction,
        the sort stable on ties; sums from _segment_sums."""
        # np.unique(components)[1:] without the sort: the labels are 1..n_lab,
        # and "[1:]" drops label 1 too when no voxel is background
        labels = np.arange(1 if has_background else 2, n_lab + 1)
        lengths = {}
        for lab in labels:
            lengths[lab] = np.linalg.norm(sums[lab])
        ordered = sorted(lengths, key=lambda k: lengths[k], reverse=True)
        boundary = int(np.ceil(3 * np.log(np.e + len(ordered))))
        print("Keeping %s of %s labels." % (boundary, len(ordered)))
        return ordered[:boundary]

    class _Timer(object):
        def __init__(self, timings, name):
            self.t, self.name = timings, name

        def __enter__(self):
            self.t0 = time.perf_counter()

        def __exit__(self, *exc):
            self.t[self.name] = self.t.get(self.name, 0.0) + time.perf_counter() - self.t0

    def _timed(self, name):
        if not hasattr(self, "timings"):
            self.timings = {}
        return AdvancedAdjuster._Timer(self.timings, name)

    def _label_ridge(self):
        """adjust_directions.py:258-288.  The ridge candidates and the main
        directions come from one pass over the quaternions
        (m16_detect_ridges_main_directions); the directions are kept on the
        device for _qeigs_to_main_dirs."""
        torch = N.torch_mod()
        shape = tuple(int(v) for v in self.response.shape)
        resp = N.to_device_f32(self.response, shape)
        d_ridge = torch.empty(shape, dtype=torch.float32, device=N.device())
        self._d_main = torch.empty_like(self._d_qeigs)
        st = N.lib().m16_detect_ridges_main_directions(N.ptr(resp), N.ptr(self._d_qeigs), shape[0], shape[1],
                                                      shape[2], float(self._ridge_detector.threshold),
                                                      N.ptr(d_ridge), N.ptr(self._d_main), N.stream_ptr())
        N.check("m16_detect_ridges_main_directions", st)
        ridge = np.require(d_ridge.cpu().numpy(), np.float32, ["C", "A", "W"])
        if self._hysteresis:
            sure = np.logical_and(ridge, self.response >= self.threshold[1])
            ridge[:] = hysteresis_threshold(ridge, sure, labeler=self.labeler)
        self.__ridge = ridge
        return ridge

    def _do_clean_ridge(self, labeled_ridge, ridge_coords, ridge_dirs):
        """Keep the ceil(3 ln(e + n)) 26-connected ridge segments whose summed
        directions are longest (adjust_directions.py:290-339).  Per segment the
        directions are summed in the reference's order (C order of the voxels)."""
        with self._timed("clean_labels"):
            components, n_lab = label26(labeled_ridge, where=self.labeler)
        with self._timed("clean_segment_sums"):
            point_label = components[tuple(np.asarray(ridge_coords, np.intp).T)]
            sums = self._segment_sums(point_label, n_lab, ridge_dirs)
            kept = self._kept_segments(n_lab, len(ridge_coords) < components.size, sums)
        keep = np.zeros(n_lab + 1, dtype=bool)   # np.in1d(components, kept) as a table lookup
        keep[np.asarray(kept, dtype=np.int64)] = True
        cleaned = keep[components].astype(labeled_ridge.dtype).reshape(components.shape)
        self.__ridge = cleaned
        return cleaned

    def _qeigs_to_main_dirs(self):
        """adjust_directions.py:341-362: the device quaternion buffer is
        overwritten with the main directions, which are also returned."""
        if getattr(self, "_d_main", None) is not None:   # computed with the ridge candidates
            self._d_qeigs.copy_(self._d_main)
            self._d_main = None
        else:
            n = self._d_qeigs.numel() // 3
            st = N.lib().m16_extract_main_directions(N.ptr(self._d_qeigs), n, N.ptr(self._d_qeigs),
                                                     N.stream_ptr())
            N.check("m16_extract_main_directions", st)
        main_dirs = self._d_qeigs.cpu().numpy()
        self.__main_dirs_unadjusted = main_dirs.copy()
        return main_dirs

    def _adjust_ridge_directions(self, labeled_ridge, main_dirs, join_components=True):
        """MST over the ridge points, sign propagation from point 0
        (adjust_directions.py:365-417).  Returns (coords uint16 R x 3,
        directions float32 R x 3).  The tree is SciPy's Kruskal tree with
        equal distances taken in (i, j) order, computed without the dense
        distance matrix (ridge_mst.py).  join_components=False leaves out the
        MST edges between groups of points more than one step apart, so each
        group keeps its own global sign; the cleaning only uses per-segment
        norms of sums, which that sign does not change."""
        with self._timed("ridge_coordinates"):
            coords = np.argwhere(labeled_ridge)   # C order, as zip(*np.where(...))
        if len(coords) == 0:
            raise ValueError("no ridge points: nothing to propagate directions along")
        with self._timed("mst_local" if not join_components else "mst_local_and_joins"):
            a, b = ridge_mst_edges(coords, self.voxel_size, join_components=join_components, local=self.mst_local)
        with self._timed("sign_propagation"):
            dirs = main_dirs[coords[:, 0], coords[:, 1], coords[:, 2]]
            adjusted = propagate_signs(len(coords), a, b, dirs)
        return np.asarray(coords, dtype=np.uint16, order="C"), adjusted

    def _adjust_all_directions(self, ridge_coords, ridge_dirs):
        """Nearest-ridge sign flip of every voxel on the GPU
        (adjust_directions.py:419-446)."""
        torch = N.torch_mod()
        assert len(ridge_coords) == len(ridge_dirs)
        # uint16 coordinates travel as int16 (same bits; the kernel reads uint16)
        coords = torch.from_numpy(np.ascontiguousarray(ridge_coords, dtype=np.uint16).view(np.int16)).to(N.device())
        rdirs = N.to_device_f32(ridge_dirs)
        d0, d1, d2 = self.response.shape
        sc = (ctypes.c_double * 3)(*[float(v) for v in self.voxel_size])
        L = N.lib()
        ws = N.workspace(L.m16_adjust_nonridge_signs_workspace_bytes(d0, d1, d2, len(ridge_coords)))
        st = L.m16_adjust_nonridge_signs_indexed(N.ptr(self._d_qeigs), d0, d1, d2, N.ptr(coords), N.ptr(rdirs),
                                                 len(ridge_coords), sc, N.ptr(ws), ws.numel(), N.stream_ptr())
        N.check("m16_adjust_nonridge_signs_indexed", st)
        return self._d_qeigs.cpu().numpy()


class TransformationCompleter(TreePrintable):
    """adjust_directions.py:449-517: complete each vector to a right-handed
    orthonormal frame and return its squeezed quaternion."""

    def __init__(self, dirs, loader=None):
        self.__dirs = None
        self._dtype = np.float32
        self._loader = loader  # accepted for compatibility, unused
        if dirs is not None:
            self.dirs = dirs

    def complete(self):
        torch = N.torch_mod()
        on_device = N.is_torch(self.__dirs)
        d = N.to_device_f32(self.__dirs)
        out = torch.empty_like(d)
        st = N.lib().m16_complete_transformations(N.ptr(d), d.numel() // 3, N.ptr(out), N.stream_ptr())
        N.check("m16_complete_transformations", st)
        return out if on_device else out.cpu().numpy()

    @property
    def dirs(self):
        return self.__dirs

    @dirs.setter
    def dirs(self, value):
        self.__dirs = value if N.is_torch(value) else np.require(value, dtype=self._dtype, requirements=["C", "A"])
