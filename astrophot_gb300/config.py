"""Global configuration mirroring ``astrophot/AP_config.py:7-66``.

Parameters and images are float64 host tensors (``ap_dtype``); the CUDA kernels receive
float32 pixels and float64 parameters.  ``ap_device`` names the GPU the kernels run on.
"""

import logging

import torch

ap_dtype = torch.float64
ap_device = "cuda:0"
ap_verbose = 0
ap_logger = logging.getLogger("astrophot_gb300")
if not ap_logger.handlers:
    ap_logger.addHandler(logging.NullHandler())


def set_logging_output(stdout=True, filename=None, **kwargs):
    ap_logger.handlers = []
    ap_logger.setLevel(logging.INFO)
    if stdout:
        ap_logger.addHandler(logging.StreamHandler())
    if filename is not None:
        ap_logger.addHandler(logging.FileHandler(filename))
