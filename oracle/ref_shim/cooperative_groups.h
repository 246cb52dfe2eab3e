// Host stand-in for <cooperative_groups.h>: enough of the cluster API for the
// reference's get_mapped_block and kernel body to compile as host code.
// refhost_driver.cpp never calls the kernel; get_mapped_block is not used either.
// TEST INFRASTRUCTURE.
#pragma once
namespace cooperative_groups {
struct cluster_group {
  template <class T> T* map_shared_rank(T* p, unsigned) const { return p; }
  unsigned block_rank() const { return 0; }
  unsigned num_threads() const { return 0; }
  unsigned thread_rank() const { return 0; }
  void sync() const {}
};
struct grid_group {
  unsigned cluster_rank() const { return 0; }
};
static inline cluster_group this_cluster() { return cluster_group{}; }
static inline grid_group this_grid() { return grid_group{}; }
}  // namespace cooperative_groups
