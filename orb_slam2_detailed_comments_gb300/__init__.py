"""GB300-native ORB-SLAM2 feature front-end.

The compute path is liborbgpu.so (hand-written CUDA kernels for sm_103a
behind the C ABI in include/orbgpu.h); this package mirrors the reference's
ORBextractor / ORBmatcher / Frame interfaces on top of it.  There is no CPU
fallback: without the built library or a CUDA device every call raises.
"""
from ._lib import (FRAME_MAPPOINT_DTYPE, FRUSTUM_FRAME_DTYPE, KEYPOINT_DTYPE, MAPPOINT_DTYPE,  # noqa: F401
                   MAPPOINT_GEOMETRY_DTYPE, OrbGpuError, lib)
from .extractor import ORBextractor  # noqa: F401
from .matcher import ORBmatcher, FrameView, compute_stereo_matches  # noqa: F401
from .mappoints import compute_distinctive_descriptors, observations_to_csr  # noqa: F401
from .frustum import compute_image_bounds, frustum_frame, is_in_frustum, undistort_keypoints  # noqa: F401
from .bow import Vocabulary, search_by_bow, search_for_triangulation  # noqa: F401
