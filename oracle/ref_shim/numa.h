/*
 * Single-node stand-in for the six libnuma calls that Grazelle's
 * source/numanodes.c makes (numanodes.c:57,88,147,190,213,222).
 *
 * Test infrastructure only: used to compile the unmodified reference into
 * oracle/_ref/ on a machine without libnuma.  One NUMA node holding every
 * online CPU; memory comes from anonymous mmap (zero-filled, like
 * numa_alloc_onnode).  Affects allocation placement only, never results.
 */
#ifndef GRZ_REF_SHIM_NUMA_H
#define GRZ_REF_SHIM_NUMA_H

#include <stddef.h>

int numa_num_configured_nodes(void);
int numa_num_configured_cpus(void);
int numa_node_of_cpu(int cpu);
void* numa_alloc_onnode(size_t size, int node);
void numa_free(void* mem, size_t size);
void numa_tonode_memory(void* mem, size_t size, int node);

#endif
