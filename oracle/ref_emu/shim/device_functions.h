/* Empty stand-in for the CPU emulation of the archived kernels. */
