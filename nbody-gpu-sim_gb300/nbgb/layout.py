"""numpy views of the reference's binary records."""
import numpy as np

# nbody::OctreeNode (include/nbody/barnes_hut_tree.hpp:9-30), 76 bytes:
# center 0, half_size 12, center_of_mass 16, total_mass 28, children 32,
# particle_index 64, is_leaf 68, particle_count 72.
NODE_DTYPE = np.dtype([
    ("center", np.float32, 3), ("half", np.float32), ("com", np.float32, 3),
    ("mass", np.float32), ("children", np.int32, 8), ("particle_index", np.int32),
    ("is_leaf", np.uint8), ("pad", np.uint8, 3), ("particle_count", np.int32)])
assert NODE_DTYPE.itemsize == 76
