/*
 * The reference's GPU library (kronmult_gpu/kronmult.cu) compiled unmodified for
 * sm_103a into a cubin, so that the kernel this project replaces can be run on the
 * same GPU as a comparator (oracle/ref_gpu.py loads it with the CUDA driver API).
 *
 * TEST INFRASTRUCTURE ONLY.  The include path is given by oracle/Makefile.  The
 * reference's kronmult_batched<double|float> specialisations instantiate its kernel
 * template cuda_kronmult_batchelement<double|float>.
 */
#include "kronmult.cu"
