// Frame entry points (filled in with the transport kernels).
#include "context.h"

namespace kdn {
struct FrameState {};
void Context::releaseFrame() {
	delete frame;
	frame = nullptr;
}
} // namespace kdn

extern "C" {
kdn_status kdn_render(kdn_ctx*, const kdn_frame*, float*) { return KDN_NOT_READY; }
kdn_status kdn_render_device(kdn_ctx*, const kdn_frame*, float*, void*) { return KDN_NOT_READY; }
kdn_status kdn_frame_stats_get(kdn_ctx*, kdn_frame_stats*) { return KDN_NOT_READY; }
}
