"""pisco4cmb_gb300 -- GB300-native pixel-space polarized-beam convolver.

A drop-in for the convolution path of PISCO (pafluxa/pisco4cmb): Scan
pointing, Sky I/Q/U/V HEALPix maps and PolBeam Stokes beam maps in, detector
a/b time-ordered data out; and the binned map-maker that turns TOD back into
I, Q, U maps (SkyMap).  The compute path is libpisco_gb300.so
(hand-written sm_103a CUDA behind a C ABI, include/pisco_gb300.h); this
package is its host-side mirror of the reference API.
"""
from .api import (Convolver, GPUConvolver, PiscoError, PiscoInvalidArgument, PolBeam,  # noqa: F401
                  RunConfig, Scan, Sky, SkyMap, ang2pix, beam_npix_for_radius,
                  focal_plane_to_sky, gaussian_beam_param_grad, pix2ang)

__all__ = ["Convolver", "GPUConvolver", "PiscoError", "PiscoInvalidArgument", "PolBeam",
           "RunConfig", "Scan", "Sky", "SkyMap", "ang2pix", "beam_npix_for_radius",
           "focal_plane_to_sky", "gaussian_beam_param_grad", "pix2ang"]
