// os_blocked.cuh — temporally blocked red/black projection and Jacobi
// diffusion (placeholder: the plain per-sweep kernels are used until the
// blocked engine is enabled for a handle).
#pragma once

namespace osg {

inline int choose_block_k(const os_handle* h) {
  return h->cfg.projection_block > 0 ? h->cfg.projection_block : -1;
}

template <class S, class A>
inline bool blocked_supported(const os_handle*) { return false; }

template <class S, class A>
inline int enqueue_blocked_diffusion(os_handle*, cudaStream_t) { return 0; }

template <class S, class A>
inline int enqueue_blocked_projection(os_handle*, cudaStream_t) { return 0; }

}  // namespace osg
