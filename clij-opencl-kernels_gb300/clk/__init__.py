"""clk: GB300-native drop-in for CLIJ's neighbourhood-filter OpenCL kernels.

``execute`` launches one reference kernel by name with named parameters;
the pyclesperanto-style functions orchestrate whole filters.  Everything
runs through libclk_gb300.so (include/clk.h); there is no CPU fallback.
"""
from ._lib import ClkError, load  # noqa: F401
from .api import Batch, Server, op_kernel, op_morphology, op_separable  # noqa: F401
from .api import (dilate_box, dilate_sphere, erode_box, erode_sphere, execute, gaussian_blur,  # noqa: F401
                  kernel_names, launch_count, morphology, maximum_box, mean_box, median_box, median_sphere, minimum_box,
                  separable, sigma_to_n, sobel, supported, torch_dtype, version, dtype_code, image_of)
from .api import (convolve, copy, gradient, greater_constant, laplace, maximum_sphere, mean_sphere,  # noqa: F401
                  minimum_sphere)
