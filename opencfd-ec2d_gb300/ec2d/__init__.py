"""ec2d -- host side of the GB300-native OpenCFD-EC2D pseudo-time-marching core.

``ec2d.inputs``  control.in / bc2d_1.in / Mesh2d.dat / Residual.dat formats
``ec2d.grids``   synthetic grids in the reference's multi-block layout
``ec2d.gpu``     ctypes binding of the C-ABI library libec2d_gpu.so
"""
from .inputs import Params, Block  # noqa: F401
