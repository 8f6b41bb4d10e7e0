/* Empty stand-in: the emulated archived kernels take their random numbers
 * from a buffer and never call the cuRAND device API. */
