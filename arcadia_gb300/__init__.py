"""GB300-native 64-tree DDA voxel ray traversal (primary G-buffer + GI rays + SHARC + NRC)."""
