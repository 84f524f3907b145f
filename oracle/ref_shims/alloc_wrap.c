/*
 * Zero-filled aligned allocation for oracle/_ref.  The reference allocates
 * every array with _mm_malloc (src/vars.c:166-300) and reads some cells before
 * writing them (the ghost ring's edges and corners before the first halo
 * exchange; the elastic scratch `f` in elastic.c; `lambda` when
 * ANISOTROPIC == 0).  Large glibc allocations come from fresh zero pages; this
 * wrapper (linked with -Wl,--wrap=posix_memalign) makes every size behave the
 * same way, so the reference is deterministic.  Test infrastructure.
 */
#include <stdlib.h>
#include <string.h>

int __real_posix_memalign(void **ptr, size_t align, size_t size);

int __wrap_posix_memalign(void **ptr, size_t align, size_t size) {
  int rc = __real_posix_memalign(ptr, align, size);
  if (rc == 0 && *ptr) memset(*ptr, 0, size);
  return rc;
}
