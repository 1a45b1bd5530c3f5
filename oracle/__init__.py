"""CPU oracle of the voxelize -> mipmap -> cone-trace path (test infrastructure only)."""
