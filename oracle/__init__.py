"""FP64 CPU oracle for the voxel SIMP hot path (test infrastructure, never product code)."""
