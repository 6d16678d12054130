/*
 * Single-node implementation of the libnuma subset declared in numa.h.
 * Test infrastructure only (see numa.h).
 */
#include "numa.h"

#include <sys/mman.h>
#include <unistd.h>

int numa_num_configured_nodes(void) { return 1; }

int numa_num_configured_cpus(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

int numa_node_of_cpu(int cpu) { (void)cpu; return 0; }

void* numa_alloc_onnode(size_t size, int node)
{
    (void)node;
    void* p = mmap(NULL, size ? size : 1, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    return p == MAP_FAILED ? NULL : p;
}

void numa_free(void* mem, size_t size)
{
    if (mem) munmap(mem, size ? size : 1);
}

void numa_tonode_memory(void* mem, size_t size, int node) { (void)mem; (void)size; (void)node; }
