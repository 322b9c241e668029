// A driver of the reference renderer's own frame loop with the backend/gb300
// binding (kodanuki_gb300/reference_plugin/backend_gb300.cpp), compiled and
// run by tests/test_plugin_contract.py against the reference built from its
// sources: the frame is drawn as the reference's contract test draws its
// backends' frames (target/tests/generic.cpp:131 drawnWith: rendererOf, the
// Backend plugins set, rendered), and written as a PFM.
//
//   plugin_contract <scene.sdf> <cpu|gb300> [reference flags ...]
// prints: steps <n> blocks <n> device <0|1> cells <n>
#include "core/options.h"
#include "core/plugin.h"
#include "core/render.h"

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace kodanuki {
Plugin backendGb300Plugin();
void gb300Seen(std::uint64_t* steps, int* blocks, int* device, std::uint64_t* cells);
Plugin pluginNamed(const std::string& name);
} // namespace kodanuki

int main(int argc, char** argv) {
	using namespace kodanuki;
	if (argc < 3) {
		std::fprintf(stderr, "usage: plugin_contract <scene.sdf> <cpu|gb300> [flags]\n");
		return 2;
	}
	std::vector<std::string> words = { "plugin_contract", argv[1] };
	for (int i = 3; i < argc; ++i) words.push_back(argv[i]);
	std::vector<char*> values;
	for (std::string& word : words) values.push_back(word.data());
	const CommandLine arguments = { .count = int(values.size()), .values = values.data() };
	SceneFile file              = sceneOrExit(words[1]);
	const Options options       = readOptions(file, arguments, false);
	Renderer renderer           = rendererOf(std::move(file), options);
	if (std::string(argv[2]) == "gb300") renderer.backends = { backendGb300Plugin() };
	rendered(renderer);
	std::uint64_t steps = 0, cells = 0;
	int blocks = 0, device = 0;
	gb300Seen(&steps, &blocks, &device, &cells);
	std::printf("steps %llu blocks %d device %d cells %llu\n", (unsigned long long) steps, blocks, device, (unsigned long long) cells);
	return 0;
}
