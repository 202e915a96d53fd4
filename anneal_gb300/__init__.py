"""anneal_gb300: GB300-native voxel SIMP hot path (hex8 FEM solve, sensitivity, density
filter, OC update, marching cubes) behind the anneal ``simp`` / ``FEM`` interfaces."""
__version__ = "0.1.0"
