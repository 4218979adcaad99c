// Serial stand-in for the reference's Utility/ParallelScan.h ComputeOffset:
// with one emulated thread at a time in (block, thread) order, the block
// scan + atomicAdd reduces to handing out the running total to every
// thread with a non-zero element (-1 otherwise), which is the offset the
// reference computes for that thread.
#pragma once
template <int threadBlock>
inline int ComputeOffset(unsigned int element, unsigned int *sum) {
  if (element == 0) return -1;
#ifdef SHIM_OMP  // blocks on several host threads: the same offsets, in racing order
  return (int)__atomic_fetch_add(sum, element, __ATOMIC_RELAXED);
#else
  unsigned int o = *sum;
  *sum = o + element;
  return (int)o;
#endif
}
