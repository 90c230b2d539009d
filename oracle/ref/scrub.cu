// Zeroes the shared memory of every SM: launched with one maximal block per
// SM before a reference-kernel launch, so that the reference's visited-set
// filter (`__shared__ uint data[SIZE]`, graph_search.cuh:88, which the
// reference never clears) starts empty.  Built by oracle/ref/Makefile.
extern "C" __global__ void scrub_smem(unsigned nwords) {
  extern __shared__ unsigned s[];
  for (unsigned i = threadIdx.x; i < nwords; i += blockDim.x) s[i] = 0u;
  __syncthreads();
}
