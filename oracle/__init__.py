"""The oracle: CPU restatements of the reference's cloth step, LBVH and spring
topology (visg_oracle.cpp), the loader of the reference's own kernels (refkern/),
and their ctypes wrappers (ffi.py).  Test infrastructure only: the shipped library
never imports this package."""
