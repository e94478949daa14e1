"""CPU oracle for the ARAP / embedded-deformation hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy/scipy, the
reference viewer's CPU path for the deformation frame so that the CUDA
library can be checked against it.  Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline legs of ``bench.py`` may import it; the product path never
does.

Parity status: the reference cannot be compiled here (it needs Eigen 3, the
SIBR/OpenGL headers and the un-vendored CudaRasterizer), and it ships no
tests or golden outputs.  The SH-rotation matrices are pinned against the
reference's own formulas (``tests/golden/sh_rotation.json``, generated by
evaluating the formula text of cudakdtree.cu); everything else is a
line-by-line restatement whose parity is UNPINNED against executed reference
code.

Modules:
  ed     -- kNN weights, node graph, Gauss-Newton ED solve, ED blend
            (Deform.hpp, Deform.cpp)
  skin   -- 6-endpoint Gaussian refit, polar split, quaternions, SH rotation,
            sample skinning (GaussianView.cpp, helper.cpp, cudakdtree.cu)
  grid   -- scene AABB, cell binning CSR, grid samples, adaptive low-pass,
            density sampling (GaussianView.cpp, cudakdtree.cu)
  targets-- control-target generators (GaussianView.cpp, helper.cpp)
  ply    -- 3DGS PLY load/save (GaussianView.cpp)
  stage2 -- the project's definition of the Stage-II alignment step (the
            external kernels' source is absent) and the visible host
            routines JudgeEmptyGrid / ExpandOpRange (GaussianView.cpp)
  raster -- the published 3D Gaussian splatting forward, standing in for
            the un-vendored rasteriser the viewer draws with
"""
