// Plugin registry for the oracle build of the reference renderer: the same
// list the reference build generates, minus the window sink, the flight
// source and execution/packets, which are not compiled here.
#include "core/plugin.h"
#include "plugins/backend/cpu/plugin.h"
#include "plugins/build/cut_long_programs/plugin.h"
#include "plugins/build/face_slabs/plugin.h"
#include "plugins/build/faced_hits/plugin.h"
#include "plugins/build/shared_coefficients/plugin.h"
#include "plugins/build/shared_subtrees/plugin.h"
#include "plugins/build/split_beside_finer/plugin.h"
#include "plugins/detail/focus_on_view/plugin.h"
#include "plugins/detail/pilot/plugin.h"
#include "plugins/detail/split_crowded_leaves/plugin.h"
#include "plugins/detail/split_hidden_primitives/plugin.h"
#include "plugins/execution/single/plugin.h"
#include "plugins/feature/absorption/plugin.h"
#include "plugins/feature/atmosphere/plugin.h"
#include "plugins/feature/clouds/plugin.h"
#include "plugins/feature/coats/plugin.h"
#include "plugins/feature/dispersion/plugin.h"
#include "plugins/feature/path_rules/plugin.h"
#include "plugins/feature/scattering/plugin.h"
#include "plugins/feature/sky_layers/plugin.h"
#include "plugins/geometry/sphere_trace/plugin.h"
#include "plugins/geometry/tree/plugin.h"
#include "plugins/observer/metrics/plugin.h"
#include "plugins/observer/progress/plugin.h"
#include "plugins/reconstruction/atrous/plugin.h"
#include "plugins/reconstruction/mean/plugin.h"
#include "plugins/reconstruction/temporal/plugin.h"
#include "plugins/reconstruction/upsample/plugin.h"
#include "plugins/reconstruction/upscale/plugin.h"
#include "plugins/sampler/each_lamp_first/plugin.h"
#include "plugins/sampler/glowing_surfaces/plugin.h"
#include "plugins/sampler/highlight_guide/plugin.h"
#include "plugins/sampler/sky_map/plugin.h"
#include "plugins/sampler/sobol/plugin.h"
#include "plugins/sampler/toward_mirrors/plugin.h"
#include "plugins/sink/file/plugin.h"
#include "plugins/sink/frames/plugin.h"
#include "plugins/source/scene/plugin.h"
#include "plugins/stopping/confidence_interval/plugin.h"
#include "plugins/stopping/fixed_count/plugin.h"
#include "plugins/strategy/connect/plugin.h"
#include "plugins/strategy/join/plugin.h"
#include "plugins/transport/paths/plugin.h"
#include <vector>
namespace kodanuki {
std::vector<Plugin> everyPlugin() {
	return {
		backendCpuPlugin(),
		buildCutLongProgramsPlugin(),
		buildFaceSlabsPlugin(),
		buildFacedHitsPlugin(),
		buildSharedCoefficientsPlugin(),
		buildSharedSubtreesPlugin(),
		buildSplitBesideFinerPlugin(),
		detailFocusOnViewPlugin(),
		detailPilotPlugin(),
		detailSplitCrowdedLeavesPlugin(),
		detailSplitHiddenPrimitivesPlugin(),
		executionSinglePlugin(),
		featureAbsorptionPlugin(),
		featureAtmospherePlugin(),
		featureCloudsPlugin(),
		featureCoatsPlugin(),
		featureDispersionPlugin(),
		featurePathRulesPlugin(),
		featureScatteringPlugin(),
		featureSkyLayersPlugin(),
		geometrySphereTracePlugin(),
		geometryTreePlugin(),
		observerMetricsPlugin(),
		observerProgressPlugin(),
		reconstructionAtrousPlugin(),
		reconstructionMeanPlugin(),
		reconstructionTemporalPlugin(),
		reconstructionUpsamplePlugin(),
		reconstructionUpscalePlugin(),
		samplerEachLampFirstPlugin(),
		samplerGlowingSurfacesPlugin(),
		samplerHighlightGuidePlugin(),
		samplerSkyMapPlugin(),
		samplerSobolPlugin(),
		samplerTowardMirrorsPlugin(),
		sinkFilePlugin(),
		sinkFramesPlugin(),
		sourceScenePlugin(),
		stoppingConfidenceIntervalPlugin(),
		stoppingFixedCountPlugin(),
		strategyConnectPlugin(),
		strategyJoinPlugin(),
		transportPathsPlugin(),
	};
}
}
