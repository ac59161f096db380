"""GB300-native occupancy discovery, XF inter-CTA barrier and persistent
graph kernels (BFS, SSSP, MIS, colouring, BC, Boruvka MST) behind a C ABI
(include/gdb.h).  The Python layer is a thin ctypes mirror of that ABI."""
