// Serial stand-in for the reference's Utility/ParallelScan.h ComputeOffset:
// with one emulated thread at a time in (block, thread) order, the block
// scan + atomicAdd reduces to handing out the running total to every
// thread with a non-zero element (-1 otherwise), which is the offset the
// reference computes for that thread.
#pragma once
template <int threadBlock>
inline int ComputeOffset(unsigned int element, unsigned int *sum) {
  if (element == 0) return -1;
  unsigned int o = *sum;
  *sum = o + element;
  return (int)o;
}
