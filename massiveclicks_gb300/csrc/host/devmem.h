// Device memory of the library's buffers, through a per-device cache of freed
// blocks.  A fit is often created, uploaded and destroyed many times with the
// same sizes (one fit per partition, per model type, per request); cudaMalloc
// and cudaFree of its few gigabytes cost milliseconds each time, and cudaFree
// synchronises the device.  Freed blocks are kept, keyed by their rounded size,
// and handed out again; mc_empty_cache returns them to the driver.
//
// A block passed to dev_free must have no device work pending on it: callers
// synchronise (the device, or the one stream that used it) before freeing,
// as cudaFree would have done.
#ifndef MCLICKS_DEVMEM_H
#define MCLICKS_DEVMEM_H

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace mch {

// A block of at least bytes on the current device (cached if one of the same
// rounded size is free).  On an allocation failure the device's cache is
// released and the allocation retried once.
cudaError_t dev_alloc(void** p, size_t bytes);

// Returns a block from dev_alloc to its device's cache; nullptr is ignored.
void dev_free(void* p);

// Frees the cached blocks of one device (-1: every device) and returns the
// bytes released.
size_t dev_cache_release(int device);

// Bytes held in the cache of one device (-1: every device).
size_t dev_cache_bytes(int device);

// Page-locked host memory through the same kind of cache (one pool for every
// device): the readbacks of an upload go to page-locked buffers, which the
// driver copies into directly, and page-locking them anew for every model
// would cost more than the copies.  host_free returns a block to the pool;
// dev_cache_release(-1) also frees the pool's cached blocks.
cudaError_t host_alloc(void** p, size_t bytes);
void host_free(void* p);

}  // namespace mch

#endif
