"""Helpers of the GPU tests: engine adapters with the oracle's interface."""
import numpy as np

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss


class RefGpu:
    """LSS_MODE_REF engine with the RefOracle interface used by ref_cases."""

    def __init__(self, vol, dtype_code, quirk_i3=True, use_graph=True):
        self.s = lss.Segmenter(lss.MODE_REF, quirk_i3=quirk_i3, use_graph=use_graph)
        self.s.load_volume(vol)

    def set_params(self, T, eps, alpha, dt, conv=0.0):
        self.s.set_parameters(T, eps, alpha, dt, convergence_threshold=conv)

    def initialize_seed(self, x, y, z, r):
        self.s.initialize_seed((x, y, z), r)

    def step(self, k=1):
        return self.s.request_update_segmentation(k)

    @property
    def n(self):
        return self.s.get_active_element_count()

    def active(self):
        return self.s.active()

    def read_mask(self):
        return self.s.get_saveable_segmentation()

    def read_phi(self):
        return self.s.read_phi()

    def read_export(self):
        return self.s.read_export()

    def read_active_volume(self):
        return self.s.read_active_volume()

    def freeze(self):
        self.s.freeze_current_segmentation()

    def clear_current(self):
        self.s.clear_current_segmentation()

    def estimate_params(self):
        return self.s.calculate_segmentation_parameters()


def dice(a, b):
    a = a.astype(bool)
    b = b.astype(bool)
    s = a.sum() + b.sum()
    return 1.0 if s == 0 else 2.0 * (a & b).sum() / s
