// Fixture exporter over the reference renderer's own library (built from its
// sources by oracle/ref/Makefile).  It is test infrastructure: it runs only in
// the container that holds the reference checkout and writes the golden
// inputs/outputs the parity tests read.
//
//   kdn_ref_dump scene  <file.sdf> <out.json>            compiled scene as JSON
//   kdn_ref_dump trace  <file.sdf> <rays.f32> <hits.bin>  sphereTraced per ray
//   kdn_ref_dump cells  <file.sdf> <targets.u32> <out.bin> cutCell of chosen cells
//   kdn_ref_dump cut    <file.sdf> <depth> <out.bin>      cutCell down an octree
//   kdn_ref_dump denoise  <in.bin> <out.f32>              denoisedFrame
//   kdn_ref_dump temporal <in.bin> <out.bin>              temporalFrame
//   kdn_ref_dump bsdf  <file.sdf> <in.bin> <out.bin>      respondBsdf, sampleBsdf
//   kdn_ref_dump upscale  <in.bin> <out.bin>              upscaledFrame
//   kdn_ref_dump upsample <in.bin> <out.bin>              upsampledImage
//   kdn_ref_dump sobol    <in.bin> <out.f64>              sobolNumber, sobolPair
//
// Reference entry points used: loadScene (syntax/evaluator.cpp:2898),
// sceneRegion (plugins/geometry/tree/build.cpp:405), sphereTraced
// (plugins/geometry/sphere_trace/sphere_trace.cpp:216), rootPrograms/cutCell/
// octantBox/regionBox (plugins/geometry/tree/cut.cpp:463 ff).
#include "plugins/feature/dispersion/dispersion.h"
#include "plugins/geometry/sphere_trace/sphere_trace.h"
#include "plugins/geometry/tree/build.h"
#include "plugins/geometry/tree/cut.h"
#include "plugins/reconstruction/atrous/atrous.h"
#include "plugins/reconstruction/temporal/temporal.h"
#include "plugins/reconstruction/upsample/upsample.h"
#include "plugins/sampler/sobol/sobol.h"
#include "plugins/reconstruction/upscale/upscale.h"
#include "plugins/transport/paths/material/material.h"
#include "sdf/program.h"
#include "sdf/scene.h"
#include "syntax/evaluator.h"

#include <array>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace kodanuki;

namespace kodanuki {
// plugins/transport/paths/material/material.cpp:329, defined with external
// linkage there but declared in no header
Sides sidesOf(const Materials& materials, std::uint32_t material, std::uint32_t medium);
}

namespace {

SceneFile loaded(const char* path) {
	LoadedScene scene = loadScene(path, 0.0);
	if (!scene.error.empty()) {
		std::fprintf(stderr, "%s\n", scene.error.c_str());
		std::exit(1);
	}
	return scene.file;
}

void putDouble(FILE* f, double v) {
	std::fprintf(f, "%.17g", v);
}

void putVector(FILE* f, const math::Vector& v) {
	std::fprintf(f, "[%.17g,%.17g,%.17g]", v.x, v.y, v.z);
}

void putColour(FILE* f, const Colour& c) {
	std::fprintf(f, "[%.17g,%.17g,%.17g]", c.red, c.green, c.blue);
}

int dumpScene(const char* sdf, const char* out) {
	const SceneFile file = loaded(sdf);
	const Region region  = sceneRegion(file.scene, file.shot, 8);
	FILE* f              = std::fopen(out, "w");
	std::fprintf(f, "{\"region\":{\"lower\":[%.17g,%.17g,%.17g],\"size\":[%.17g,%.17g,%.17g]},\n", region.lower[0], region.lower[1], region.lower[2], region.size[0], region.size[1], region.size[2]);
	std::fprintf(f, "\"programs\":[\n");
	for (std::size_t i = 0; i < file.scene.objectPrograms.size(); ++i) {
		const Program& program = file.scene.objectPrograms[i];
		std::fprintf(f, "%s{\"result\":%u,\"steps\":[", i ? ",\n" : "", program.result);
		for (std::size_t s = 0; s < program.steps.size(); ++s) {
			const Step& step = program.steps[s];
			std::fprintf(f, "%s[%d,%u,%u,%u,%.17g,%u]", s ? "," : "", int(step.opcode), step.a, step.b, step.c, step.value, step.leaf);
		}
		std::fprintf(f, "]}");
	}
	std::fprintf(f, "],\n\"leaves\":[");
	for (std::size_t i = 0; i < file.scene.leaves.size(); ++i) {
		std::fprintf(f, "%s%u", i ? "," : "", file.scene.leaves[i].material);
	}
	// sdf/scene.h Placement of each leaf: linear (row by row), then origin
	std::fprintf(f, "],\n\"placements\":[");
	for (std::size_t i = 0; i < file.scene.leaves.size(); ++i) {
		const Placement& pl = file.scene.leaves[i].placement;
		std::fprintf(f, "%s[", i ? "," : "");
		for (int r = 0; r < 3; ++r) {
			for (int c = 0; c < 3; ++c) std::fprintf(f, "%.17g,", pl.linear[r][c]);
		}
		std::fprintf(f, "%.17g,%.17g,%.17g]", pl.origin[0], pl.origin[1], pl.origin[2]);
	}
	std::fprintf(f, "],\n\"materials\":[");
	for (std::size_t i = 0; i < file.looks.materials.size(); ++i) {
		const Material& m = file.looks.materials[i];
		std::fprintf(f, "%s{\"kind\":%d,\"stops\":[", i ? ",\n" : "", int(m.kind));
		for (std::size_t s = 0; s < m.albedo.stops.size(); ++s) {
			std::fprintf(f, "%s%.9g", s ? "," : "", double(m.albedo.stops[s]));
		}
		std::fprintf(f, "],\"pattern\":%d,\"roughness\":%.9g,\"refraction\":%.9g,\"dispersion\":%.9g,\"scatter\":%.9g,\"absorb\":", m.albedo.program, double(m.roughness), double(m.refraction), double(m.dispersion), double(m.scatter));
		putColour(f, m.absorb);
		std::fprintf(f, ",\"glow\":");
		putColour(f, m.glow);
		std::fprintf(f, ",\"strength\":%.9g,\"lean\":%.9g,\"film\":[%.9g,%.9g],\"coats\":%zu", double(m.strength), double(m.lean), double(m.film[0]), double(m.film[1]), file.looks.coats.size());
		// sdf/scene.h Albedo: the pattern's program (Scene::programs), the
		// arguments it reads (Scene::arguments from Albedo::arguments), and
		// whether it is read in world space
		std::fprintf(f, ",\"world\":%d", int(m.albedo.world));
		if (m.albedo.program >= 0) {
			const Program& program = file.scene.programs[std::size_t(m.albedo.program)];
			std::fprintf(f, ",\"patternResult\":%u,\"patternSteps\":[", program.result);
			for (std::size_t s = 0; s < program.steps.size(); ++s) {
				const Step& step = program.steps[s];
				std::fprintf(f, "%s[%d,%u,%u,%u,%.17g,%u]", s ? "," : "", int(step.opcode), step.a, step.b, step.c, step.value, step.leaf);
			}
			std::fprintf(f, "],\"patternArguments\":[");
			for (std::uint32_t k = 0; k < program.arguments; ++k) {
				std::fprintf(f, "%s%.17g", k ? "," : "", file.scene.arguments[m.albedo.arguments + k]);
			}
			std::fprintf(f, "]");
		}
		std::fprintf(f, "}");
	}
	std::fprintf(f, "],\n\"lights\":[");
	for (std::size_t i = 0; i < file.lighting.lights.size(); ++i) {
		const Light& l = file.lighting.lights[i];
		std::fprintf(f, "%s{\"kind\":%d,\"at\":", i ? ",\n" : "", int(l.kind));
		putVector(f, l.at);
		std::fprintf(f, ",\"direction\":");
		putVector(f, l.direction);
		std::fprintf(f, ",\"along\":");
		putVector(f, l.along);
		std::fprintf(f, ",\"across\":");
		putVector(f, l.across);
		std::fprintf(f, ",\"radius\":%.9g,\"angle\":%.9g,\"power\":", double(l.radius), double(l.angle));
		putColour(f, l.power);
		std::fprintf(f, "}");
	}
	// plugins/transport/paths/material/material.cpp:287 materialsOf: the finish
	// each material is drawn with, its escape table included
	const Materials made = materialsOf(file.looks, SmoothGlass::Exact);
	std::fprintf(f, "],\n\"finishes\":[");
	for (std::size_t i = 0; i < made.finishes.size(); ++i) {
		const Finish& fin = made.finishes[i];
		std::fprintf(f, "%s{\"kind\":%d,\"width\":%.17g,\"sharp\":%d,\"facetShare\":%.17g,\"body\":%.17g,\"coating\":[%.17g,%.17g,%.17g],\"index\":%.17g,\"losesMuch\":%d,\"exact\":%d,\"film\":[%.17g,%.17g],\"escapeAverage\":%.17g,\"escape\":[",
		             i ? ",\n" : "", int(fin.kind), fin.width, int(fin.sharp), fin.facetShare, fin.body, fin.coating.front, fin.coating.twice, fin.coating.room, fin.index, int(fin.losesMuch), int(fin.exact), fin.film.thickness, fin.film.index, fin.escape.average);
		for (int k = 0; k < energyViews; ++k) {
			std::fprintf(f, "%s%.17g", k ? "," : "", fin.escape.table[std::size_t(k)]);
		}
		std::fprintf(f, "]");
		// material/energy.h Boundary of a glass: rarer, denser (a row of
		// views per ratio), rarerAverage, denserAverage, rarerThrough
		if (fin.kind == MaterialKind::Glass) {
			std::fprintf(f, ",\"boundary\":[");
			bool first = true;
			const auto put = [&](const double* v, std::size_t n) {
				for (std::size_t k = 0; k < n; ++k) {
					std::fprintf(f, "%s%.17g", first ? "" : ",", v[k]);
					first = false;
				}
			};
			put(fin.boundary.rarer.data(), fin.boundary.rarer.size());
			put(fin.boundary.denser.data(), fin.boundary.denser.size());
			put(fin.boundary.rarerAverage.data(), fin.boundary.rarerAverage.size());
			put(fin.boundary.denserAverage.data(), fin.boundary.denserAverage.size());
			put(fin.boundary.rarerThrough.data(), fin.boundary.rarerThrough.size());
			std::fprintf(f, "]");
		}
		std::fprintf(f, "}");
	}
	const Sky& sky = file.lighting.sky;
	std::fprintf(f, "],\n\"sky\":{\"kind\":%d,\"zenith\":", int(sky.kind));
	putColour(f, sky.zenith);
	std::fprintf(f, ",\"horizon\":");
	putColour(f, sky.horizon);
	std::fprintf(f, ",\"ground\":");
	putColour(f, sky.ground);
	std::fprintf(f, ",\"glow\":");
	putColour(f, sky.glow);
	std::fprintf(f, ",\"strength\":%.9g,\"spread\":%.9g,\"haze\":%.9g", double(sky.strength), double(sky.spread), double(sky.haze));
	const Stars& stars = file.lighting.stars;
	std::fprintf(f, ",\"stars\":%d,\"star_count\":%.9g,\"star_strength\":%.9g,\"star_angle\":%.9g", stars.present ? 1 : 0, double(stars.count), double(stars.strength), double(stars.angle));
	const Camera& c = file.shot.camera;
	const Render& r = file.shot.render;
	std::fprintf(f, "},\n\"camera\":{\"eye\":");
	putVector(f, c.eye);
	std::fprintf(f, ",\"target\":");
	putVector(f, c.target);
	std::fprintf(f, ",\"up\":");
	putVector(f, c.up);
	std::fprintf(f, ",\"fov\":%.9g,\"aperture\":%.9g,\"focus\":%.9g},\n", double(c.fov), double(c.aperture), double(c.focus));
	std::fprintf(f, "\"render\":{\"width\":%d,\"height\":%d,\"seed\":%d,\"samples\":%d,\"surfaces\":%d,\"collisions\":%d,\"split\":%d,\"far\":", r.width, r.height, r.seed, r.samples, r.surfaces, r.collisions, r.split);
	putDouble(f, r.far);
	std::fprintf(f, "}}\n");
	std::fclose(f);
	return 0;
}

// Rays: float32 records of 8 (origin xyz, direction xyz, far, inside) plus the
// reference region; hits: per ray {kind u32, distance f32, point f32x3,
// normal f32x3, leaf u32, other u32, share f32} = 44 bytes.
int dumpTrace(const char* sdf, const char* raysPath, const char* hitsPath) {
	const SceneFile file = loaded(sdf);
	const Region region  = reachRegion(file.shot);
	const Geometry geo   = sphereGeometry(file.scene, region);
	FILE* in             = std::fopen(raysPath, "rb");
	std::vector<float> rays;
	float record[8];
	while (std::fread(record, sizeof(float), 8, in) == 8) {
		rays.insert(rays.end(), record, record + 8);
	}
	std::fclose(in);
	FILE* out = std::fopen(hitsPath, "wb");
	for (std::size_t i = 0; i < rays.size(); i += 8) {
		const Ray ray = {
			.origin    = { rays[i], rays[i + 1], rays[i + 2] },
			.direction = { rays[i + 3], rays[i + 4], rays[i + 5] },
			.far       = rays[i + 6],
			.inside    = rays[i + 7] != 0,
			.within    = noMaterial,
		};
		const Hit hit           = sphereTraced(geo, ray);
		const std::uint32_t u[] = { std::uint32_t(hit.kind) };
		std::fwrite(u, 4, 1, out);
		const float g[] = { hit.distance, hit.point.x, hit.point.y, hit.point.z, hit.normal.x, hit.normal.y, hit.normal.z };
		std::fwrite(g, 4, 7, out);
		const std::uint32_t ids[] = { hit.leaf, hit.other };
		std::fwrite(ids, 4, 2, out);
		std::fwrite(&hit.share, 4, 1, out);
	}
	std::fclose(out);
	return 0;
}

struct CutWriter {
	FILE* out;
	int depth;
	std::uint64_t leaves;
};

// Per visited cell (pre-order): level u32, place xyz u32, occupancy u32,
// object count u32, then per object: object u32, result u32, step count u32,
// steps (opcode u32, a, b, c u32, value f64, leaf u32).  A surface cell above
// the depth is split into its eight octants and recursed.
void writeCell(CutWriter& writer, const CellPrograms& programs, const Box& box, int level, const std::uint32_t place[3]) {
	const CellCut cut       = cutCell(programs, box);
	const std::uint32_t h[] = { std::uint32_t(level), place[0], place[1], place[2], std::uint32_t(cut.occupancy), std::uint32_t(cut.programs.objects.size()) };
	std::fwrite(h, 4, 6, writer.out);
	for (std::size_t i = 0; i < cut.programs.objects.size(); ++i) {
		const Program& program  = *cut.programs.programs[i];
		const std::uint32_t o[] = { cut.programs.objects[i], program.result, std::uint32_t(program.steps.size()) };
		std::fwrite(o, 4, 3, writer.out);
		for (const Step& step : program.steps) {
			const std::uint32_t s[] = { std::uint32_t(step.opcode), step.a, step.b, step.c };
			std::fwrite(s, 4, 4, writer.out);
			std::fwrite(&step.value, 8, 1, writer.out);
			std::fwrite(&step.leaf, 4, 1, writer.out);
		}
	}
	++writer.leaves;
	if (cut.occupancy != Occupancy::Surface || level >= writer.depth) {
		return;
	}
	for (int octant = 0; octant < 8; ++octant) {
		const std::uint32_t child[3] = { place[0] * 2 + (octant & 1), place[1] * 2 + ((octant >> 1) & 1), place[2] * 2 + ((octant >> 2) & 1) };
		writeCell(writer, cut.programs, octantBox(box, octant), level + 1, child);
	}
}

int dumpCut(const char* sdf, int depth, const char* outPath) {
	const SceneFile file = loaded(sdf);
	const Region region  = sceneRegion(file.scene, file.shot, 8);
	CutWriter writer     = { std::fopen(outPath, "wb"), depth, 0 };
	const std::uint32_t root[3] = { 0, 0, 0 };
	writeCell(writer, rootPrograms(file.scene), regionBox(region), 0, root);
	std::fclose(writer.out);
	std::fprintf(stderr, "%llu cells\n", (unsigned long long) writer.leaves);
	return 0;
}

// The reference's cut of chosen cells: each target (level, place) is reached
// from the root by cutting every cell on its path (a child is cut from its
// parent's cut, as writeCell does), the paths' common cells cut once.
struct Target {
	std::uint32_t level, place[3];
	std::size_t index;
};

void cutTargets(const CellPrograms& programs, const Box& box, std::uint32_t level, const std::uint32_t place[3], std::vector<Target> targets,
                std::vector<std::vector<std::uint8_t>>& records) {
	const CellCut cut = cutCell(programs, box);
	std::vector<Target> below;
	for (const Target& t : targets) {
		if (t.level != level) {
			below.push_back(t);
			continue;
		}
		std::vector<std::uint8_t>& rec = records[t.index];
		auto put = [&](const void* p, std::size_t n) { rec.insert(rec.end(), static_cast<const std::uint8_t*>(p), static_cast<const std::uint8_t*>(p) + n); };
		const std::uint32_t h[] = { level, place[0], place[1], place[2], std::uint32_t(cut.occupancy), std::uint32_t(cut.programs.objects.size()) };
		put(h, sizeof h);
		for (std::size_t i = 0; i < cut.programs.objects.size(); ++i) {
			const Program& program  = *cut.programs.programs[i];
			const std::uint32_t o[] = { cut.programs.objects[i], program.result, std::uint32_t(program.steps.size()) };
			put(o, sizeof o);
			for (const Step& step : program.steps) {
				const std::uint32_t st[] = { std::uint32_t(step.opcode), step.a, step.b, step.c };
				put(st, sizeof st);
				put(&step.value, 8);
				put(&step.leaf, 4);
			}
		}
	}
	for (int octant = 0; octant < 8; ++octant) {
		const std::uint32_t child[3] = { place[0] * 2 + (octant & 1), place[1] * 2 + ((octant >> 1) & 1), place[2] * 2 + ((octant >> 2) & 1) };
		std::vector<Target> mine;
		for (const Target& t : below) {
			const std::uint32_t shift = t.level - level - 1;
			if ((t.place[0] >> shift) == child[0] && (t.place[1] >> shift) == child[1] && (t.place[2] >> shift) == child[2]) mine.push_back(t);
		}
		if (!mine.empty()) cutTargets(cut.programs, octantBox(box, octant), level + 1, child, mine, records);
	}
}

// targets file: u32 count, then (level, x, y, z) u32 each; output: one
// writeCell record a target, in the targets' order (no recursion below it).
int dumpCells(const char* sdf, const char* targetsPath, const char* outPath) {
	const SceneFile file = loaded(sdf);
	const Region region  = sceneRegion(file.scene, file.shot, 8);
	FILE* in             = std::fopen(targetsPath, "rb");
	std::uint32_t count  = 0;
	if (std::fread(&count, 4, 1, in) != 1) return 1;
	std::vector<Target> targets(count);
	for (std::uint32_t i = 0; i < count; ++i) {
		std::uint32_t v[4];
		if (std::fread(v, 4, 4, in) != 4) return 1;
		targets[i] = Target { v[0], { v[1], v[2], v[3] }, i };
	}
	std::fclose(in);
	std::vector<std::vector<std::uint8_t>> records(count);
	const std::uint32_t root[3] = { 0, 0, 0 };
	cutTargets(rootPrograms(file.scene), regionBox(region), 0, root, targets, records);
	FILE* out = std::fopen(outPath, "wb");
	for (const auto& r : records) std::fwrite(r.data(), 1, r.size(), out);
	std::fclose(out);
	return 0;
}

// Feature buffers in, the reference's denoised frame out
// (plugins/reconstruction/atrous/atrous.cpp:513 denoisedFrame).  Input: int32
// width, height, demodulated; doubles eye[3], forward[3], right[3], up[3],
// reach, aspect; then per pixel colour[3] f64, moment f64, length f32,
// distance f32, normal[3] f64, leaf u32, albedo[3] f64.  Output: RGB f32.
int dumpDenoise(const char* inPath, const char* outPath) {
	FILE* in = std::fopen(inPath, "rb");
	std::int32_t head[3];
	double lensValues[14];
	if (std::fread(head, 4, 3, in) != 3 || std::fread(lensValues, 8, 14, in) != 14) return 1;
	TemporalState temporal = emptyTemporal();
	temporal.width         = head[0];
	temporal.height        = head[1];
	temporal.demodulated   = head[2] != 0;
	for (int k = 0; k < head[0] * head[1]; ++k) {
		double colour[3], moment, normal[3], albedo[3];
		float length, distance;
		std::uint32_t leaf;
		if (std::fread(colour, 8, 3, in) != 3 || std::fread(&moment, 8, 1, in) != 1 || std::fread(&length, 4, 1, in) != 1 || std::fread(&distance, 4, 1, in) != 1 ||
		    std::fread(normal, 8, 3, in) != 3 || std::fread(&leaf, 4, 1, in) != 1 || std::fread(albedo, 8, 3, in) != 3) {
			return 1;
		}
		temporal.pixels.push_back(TemporalPixel {
			.colour   = { colour[0], colour[1], colour[2] },
			.moment   = moment,
			.length   = length,
			.distance = distance,
			.normal   = { normal[0], normal[1], normal[2] },
			.leaf     = leaf,
			.albedo   = { albedo[0], albedo[1], albedo[2] },
		});
	}
	std::fclose(in);
	const Lens lens = {
		.eye      = { lensValues[0], lensValues[1], lensValues[2] },
		.forward  = { lensValues[3], lensValues[4], lensValues[5] },
		.right    = { lensValues[6], lensValues[7], lensValues[8] },
		.up       = { lensValues[9], lensValues[10], lensValues[11] },
		.reach    = lensValues[12],
		.aspect   = lensValues[13],
		.aperture = 0,
		.focus    = 10,
		.width    = head[0],
		.height   = head[1],
	};
	static const FrameRecord record = emptyFrameRecord();
	static const std::vector<PixelSum> estimates;
	const ShownFrame frame = {
		.width     = head[0],
		.height    = head[1],
		.lens      = lens,
		.before    = lens,
		.film      = { .factor = 1, .phase = 0 },
		.moved     = false,
		.restarted = false,
		.recounted = false,
		.still     = 1,
		.record    = record,
		.estimates = estimates,
		.surfaces  = noSurfaces(),
		.threads   = 4,
	};
	const Denoised denoised = denoisedFrame(emptyDenoise(), temporal, frame);
	FILE* out               = std::fopen(outPath, "wb");
	std::fwrite(denoised.image.rgb.data(), 4, denoised.image.rgb.size(), out);
	std::fclose(out);
	return 0;
}

Lens lensOf14(const double* v, int width, int height) {
	return Lens {
		.eye      = { v[0], v[1], v[2] },
		.forward  = { v[3], v[4], v[5] },
		.right    = { v[6], v[7], v[8] },
		.up       = { v[9], v[10], v[11] },
		.reach    = v[12],
		.aspect   = v[13],
		.aperture = 0,
		.focus    = 10,
		.width    = width,
		.height   = height,
	};
}

bool readSurface(FILE* in, Surface& s) {
	float distance, normal[3], albedo[3];
	std::uint32_t leaf;
	if (std::fread(&distance, 4, 1, in) != 1 || std::fread(normal, 4, 3, in) != 3 || std::fread(&leaf, 4, 1, in) != 1 || std::fread(albedo, 4, 3, in) != 3) return false;
	s          = missedSurface();
	s.distance = distance;
	s.normal   = { normal[0], normal[1], normal[2] };
	s.leaf     = leaf;
	s.albedo   = { albedo[0], albedo[1], albedo[2] };
	return true;
}

bool readPixel(FILE* in, TemporalPixel& p) {
	double colour[3], moment, normal[3], albedo[3];
	float length, distance;
	std::uint32_t leaf;
	if (std::fread(colour, 8, 3, in) != 3 || std::fread(&moment, 8, 1, in) != 1 || std::fread(&length, 4, 1, in) != 1 || std::fread(&distance, 4, 1, in) != 1 ||
	    std::fread(normal, 8, 3, in) != 3 || std::fread(&leaf, 4, 1, in) != 1 || std::fread(albedo, 8, 3, in) != 3) {
		return false;
	}
	p = TemporalPixel {
		.colour   = { colour[0], colour[1], colour[2] },
		.moment   = moment,
		.length   = length,
		.distance = distance,
		.normal   = { normal[0], normal[1], normal[2] },
		.leaf     = leaf,
		.albedo   = { albedo[0], albedo[1], albedo[2] },
	};
	return true;
}

void writePixel(FILE* out, const TemporalPixel& p) {
	const double colour[3] = { p.colour.red, p.colour.green, p.colour.blue };
	const double normal[3] = { p.normal.x, p.normal.y, p.normal.z };
	const double albedo[3] = { p.albedo.red, p.albedo.green, p.albedo.blue };
	std::fwrite(colour, 8, 3, out);
	std::fwrite(&p.moment, 8, 1, out);
	std::fwrite(&p.length, 4, 1, out);
	std::fwrite(&p.distance, 4, 1, out);
	std::fwrite(normal, 8, 3, out);
	std::fwrite(&p.leaf, 4, 1, out);
	std::fwrite(albedo, 8, 3, out);
}

// One frame of the temporal member (plugins/reconstruction/temporal/
// temporal.cpp:1001 temporalFrame) at a film factor of 1.  Input: int32
// width, height (the drawn grid), moved, recounted, kept (the state before
// holds a frame), demodulated (the state before's flag), film factor and
// phase, the state before's film factor and phase; doubles lens now[14], lens
// before[14] (eye, forward, right, up, reach, aspect); then per pixel the
// record's light (3 f64), the record's surface and the G-buffer's surface
// (each distance f32, normal 3 f32, leaf u32, albedo 3 f32), and the state
// before's pixel (colour 3 f64, moment f64, length f32, distance f32,
// normal 3 f64, leaf u32, albedo 3 f64).  Output: the new state's pixels
// (the same layout), then the image, RGB f32.
int dumpTemporal(const char* inPath, const char* outPath) {
	FILE* in = std::fopen(inPath, "rb");
	std::int32_t head[10];
	double now[14], before[14];
	if (std::fread(head, 4, 10, in) != 10 || std::fread(now, 8, 14, in) != 14 || std::fread(before, 8, 14, in) != 14) return 1;
	const int width = head[0], height = head[1];
	const FilmPlan film       = { .factor = head[6], .phase = head[7] };
	const FilmPlan filmBefore = { .factor = head[8], .phase = head[9] };
	const std::size_t n = std::size_t(width) * std::size_t(height);
	FrameRecord record  = emptyFrameRecord();
	record.width        = width;
	record.height       = height;
	std::vector<Surface> gbuffer(n);
	TemporalState state = emptyTemporal();
	state.width         = head[4] ? width : 0;
	state.height        = head[4] ? height : 0;
	state.demodulated   = head[5] != 0;
	state.film          = filmBefore;
	for (std::size_t k = 0; k < n; ++k) {
		double light[3];
		Surface first, centre;
		TemporalPixel last;
		if (std::fread(light, 8, 3, in) != 3 || !readSurface(in, first) || !readSurface(in, centre) || !readPixel(in, last)) return 1;
		record.parts.push_back(Parts { .total = { light[0], light[1], light[2] } });
		record.surfaces.push_back(first);
		gbuffer[k] = centre;
		if (head[4]) state.pixels.push_back(last);
	}
	std::fclose(in);
	// the shown frame: the drawn grid times the factor (core/shown.cpp:7 shownLens)
	const Lens lensNow    = lensOf14(now, width * film.factor, height * film.factor);
	const Lens lensBefore = lensOf14(before, width * film.factor, height * film.factor);
	static const std::vector<PixelSum> estimates;
	const ShownFrame frame = {
		.width     = width * film.factor,
		.height    = height * film.factor,
		.lens      = lensNow,
		.before    = lensBefore,
		.film      = film,
		.moved     = head[2] != 0,
		.restarted = false,
		.recounted = head[3] != 0,
		.still     = head[2] ? 1u : 2u,
		.record    = record,
		.estimates = estimates,
		.surfaces  = gbuffer,
		.threads   = 4,
	};
	const Temporal next = temporalFrame(state, frame);
	FILE* out           = std::fopen(outPath, "wb");
	for (const TemporalPixel& p : next.state.pixels) writePixel(out, p);
	std::fwrite(next.image.rgb.data(), 4, next.image.rgb.size(), out);
	std::fclose(out);
	return 0;
}

// The upscale member (plugins/reconstruction/upscale/upscale.cpp
// upscaledFrame) for one frame.  Input: int32 shown width, height, film
// factor, phase, moved, restarted, kept (a state before is given), the state
// before's moved flag and settling count, surfaces (the G-buffer's
// distances are given); doubles lens now[14], lens before[14] (eye,
// forward, right, up, reach, aspect); the internal image at the drawn size
// (RGB f32); the G-buffer's distance a drawn pixel (f32) where given; the
// state before's pixels at the shown size (colour 3 f64, depth f32) where
// kept.  Output: the state after's moved flag and settling count (int32),
// its pixels (the same layout), then the image, RGB f32.
int dumpUpscale(const char* inPath, const char* outPath) {
	FILE* in = std::fopen(inPath, "rb");
	std::int32_t head[10];
	double now[14], before[14];
	if (in == nullptr || std::fread(head, 4, 10, in) != 10 || std::fread(now, 8, 14, in) != 14 || std::fread(before, 8, 14, in) != 14) return 1;
	const int width = head[0], height = head[1];
	const FilmPlan film = { .factor = head[2], .phase = head[3] };
	const int drawnWidth = width / film.factor, drawnHeight = height / film.factor;
	const std::size_t drawn = std::size_t(drawnWidth) * std::size_t(drawnHeight);
	const std::size_t shown = std::size_t(width) * std::size_t(height);
	Image internal          = blankImage(drawnWidth, drawnHeight);
	if (std::fread(internal.rgb.data(), 4, drawn * 3, in) != drawn * 3) return 1;
	std::vector<Surface> surfaces;
	if (head[9]) {
		for (std::size_t k = 0; k < drawn; ++k) {
			Surface s = missedSurface();
			if (std::fread(&s.distance, 4, 1, in) != 1) return 1;
			surfaces.push_back(s);
		}
	}
	UpscaleState state = emptyUpscale();
	if (head[6]) {
		state.width  = width;
		state.height = height;
		for (std::size_t k = 0; k < shown; ++k) {
			double colour[3];
			float depth;
			if (std::fread(colour, 8, 3, in) != 3 || std::fread(&depth, 4, 1, in) != 1) return 1;
			state.pixels.push_back(UpscalePixel { .colour = { colour[0], colour[1], colour[2] }, .depth = depth });
		}
	}
	state.moved    = head[7] != 0;
	state.settling = head[8];
	std::fclose(in);
	const Lens lensNow    = lensOf14(now, width, height);
	const Lens lensBefore = lensOf14(before, width, height);
	FrameRecord record    = emptyFrameRecord();
	record.width          = drawnWidth;
	record.height         = drawnHeight;
	static const std::vector<PixelSum> estimates;
	const ShownFrame frame = {
		.width     = width,
		.height    = height,
		.lens      = lensNow,
		.before    = lensBefore,
		.film      = film,
		.moved     = head[4] != 0,
		.restarted = head[5] != 0,
		.recounted = false,
		.still     = head[4] ? 1u : 2u,
		.record    = record,
		.estimates = estimates,
		.surfaces  = surfaces,
		.threads   = 4,
	};
	const Upscaled next = upscaledFrame(state, internal, frame);
	FILE* out           = std::fopen(outPath, "wb");
	const std::int32_t tail[2] = { next.state.moved ? 1 : 0, next.state.settling };
	std::fwrite(tail, 4, 2, out);
	for (const UpscalePixel& p : next.state.pixels) {
		const double colour[3] = { p.colour.red, p.colour.green, p.colour.blue };
		std::fwrite(colour, 8, 3, out);
		std::fwrite(&p.depth, 4, 1, out);
	}
	std::fwrite(next.image.rgb.data(), 4, next.image.rgb.size(), out);
	std::fclose(out);
	return 0;
}

// The upsample member (plugins/reconstruction/upsample/upsample.cpp
// upsampledImage).  Input: int32 shown width, height, film factor; the
// drawn image (RGB f32, the shown size over the factor).  Output: the shown
// image, RGB f32.
int dumpUpsample(const char* inPath, const char* outPath) {
	FILE* in = std::fopen(inPath, "rb");
	std::int32_t head[3];
	if (in == nullptr || std::fread(head, 4, 3, in) != 3) return 1;
	const int width = head[0], height = head[1];
	const FilmPlan film = { .factor = head[2], .phase = 0 };
	Image drawn         = blankImage(width / film.factor, height / film.factor);
	if (std::fread(drawn.rgb.data(), 4, drawn.rgb.size(), in) != drawn.rgb.size()) return 1;
	std::fclose(in);
	const Lens lens    = lensOf14(std::array<double, 14> { 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 1, 1, 1 }.data(), width, height);
	FrameRecord record = emptyFrameRecord();
	record.width       = drawn.width;
	record.height      = drawn.height;
	static const std::vector<PixelSum> estimates;
	static const std::vector<Surface> none;
	const ShownFrame frame = {
		.width     = width,
		.height    = height,
		.lens      = lens,
		.before    = lens,
		.film      = film,
		.moved     = false,
		.restarted = false,
		.recounted = false,
		.still     = 1,
		.record    = record,
		.estimates = estimates,
		.surfaces  = none,
		.threads   = 4,
	};
	const Image shown = upsampledImage(drawn, frame);
	FILE* out         = std::fopen(outPath, "wb");
	std::fwrite(shown.rgb.data(), 4, shown.rgb.size(), out);
	std::fclose(out);
	return 0;
}

// plugins/sampler/sobol/sobol.cpp sobolNumber and sobolPair of keys.
// Input records: uint64 stream, uint32 index, uint32 coordinate (below
// sobolDimensions).  Output per record: double sobolNumber, then the pair
// of the coordinate rounded down to even (its first and second number).
int dumpSobol(const char* inPath, const char* outPath) {
	FILE* in  = std::fopen(inPath, "rb");
	FILE* out = std::fopen(outPath, "wb");
	if (in == nullptr || out == nullptr) return 1;
	for (;;) {
		std::uint64_t stream;
		std::uint32_t index[2];
		if (std::fread(&stream, 8, 1, in) != 1 || std::fread(index, 4, 2, in) != 2) break;
		const math::Key key = { .stream = stream, .index = index[0], .coordinate = index[1] };
		const math::Key even = { .stream = stream, .index = index[0], .coordinate = index[1] & ~std::uint64_t(1) };
		const double number       = sobolNumber(key);
		const math::UnitPair pair = sobolPair(even);
		const double values[3]    = { number, pair.u, pair.v };
		std::fwrite(values, 8, 3, out);
	}
	std::fclose(in);
	std::fclose(out);
	return 0;
}

} // namespace

// respondBsdf and sampleBsdf (plugins/transport/paths/material/material.cpp
// :1076, :1366) at chosen vertices of a scene's materials, built as the
// renderer builds them (materialsOf with exact smooth glass, no coats), the
// sides set as its trace sets them (material.cpp:328 sidesOf, then
// feature/dispersion dispersedSides and filmedSides), the wavelengths drawn
// by math/colour.cpp sampledWavelengths.  Input records: uint32 material,
// medium (0xFFFFFFFF: outside every body); double albedo[3], normal[3],
// outgoing[3], incoming[3], wavelength share, draw numbers u, v, lobe, side.
// Output per record: double value[4], density (respondBsdf of outgoing and
// incoming); uint32 found, through; double incoming[3], weight[4], density
// (sampleBsdf from the eye with the numbers).
int dumpBsdf(const char* sdf, const char* inPath, const char* outPath) {
	const SceneFile file   = loaded(sdf);
	const Materials made   = materialsOf(file.looks, SmoothGlass::Exact);
	const Dispersion bends = dispersionOf(file.looks);
	FILE* in               = std::fopen(inPath, "rb");
	FILE* out              = std::fopen(outPath, "wb");
	if (in == nullptr || out == nullptr) {
		return 1;
	}
	for (;;) {
		std::uint32_t ids[2];
		double d[17];
		if (std::fread(ids, 4, 2, in) != 2 || std::fread(d, 8, 17, in) != 17) {
			break;
		}
		const std::uint32_t material = ids[0];
		const std::uint32_t medium   = ids[1] == 0xFFFFFFFFu ? noMaterial : ids[1];
		const Wavelengths lanes      = sampledWavelengths(d[12]);
		Sides sides                  = sidesOf(made, material, medium);
		const DispersedQuery query   = {
			  .material    = material,
			  .medium      = medium,
			  .sides       = sides,
			  .wavelengths = lanes,
        };
		sides                      = dispersedSides(bends, query);
		const DispersedQuery again = {
			.material    = material,
			.medium      = medium,
			.sides       = sides,
			.wavelengths = lanes,
		};
		sides           = filmedSides(bends, again);
		const Bsdf bsdf = {
			.material = material,
			.albedo   = FloatColour(d[0], d[1], d[2]),
			.normal   = math::FloatVector(d[3], d[4], d[5]),
			.sides    = sides,
		};
		const BsdfPair pair = {
			.outgoing    = { d[6], d[7], d[8] },
			.incoming    = { d[9], d[10], d[11] },
			.wavelengths = lanes,
		};
		const Response answer = respondBsdf(made, bsdf, pair);
		const BsdfDraw draw   = {
			  .outgoing    = { d[6], d[7], d[8] },
			  .travel      = Travel::FromEye,
			  .numbers     = { .pair = { .u = d[13], .v = d[14] }, .lobe = d[15], .side = d[16] },
			  .wavelengths = lanes,
        };
		const Scatter drawn        = sampleBsdf(made, bsdf, draw);
		const std::uint32_t seen[2] = { drawn.found ? 1u : 0u, drawn.through ? 1u : 0u };
		const double incoming[3]   = { drawn.incoming.x, drawn.incoming.y, drawn.incoming.z };
		std::fwrite(answer.value.values, 8, 4, out);
		std::fwrite(&answer.density, 8, 1, out);
		std::fwrite(seen, 4, 2, out);
		std::fwrite(incoming, 8, 3, out);
		std::fwrite(drawn.weight.values, 8, 4, out);
		std::fwrite(&drawn.density, 8, 1, out);
	}
	std::fclose(in);
	std::fclose(out);
	return 0;
}

int main(int argc, char** argv) {
	if (argc >= 4 && std::strcmp(argv[1], "temporal") == 0) {
		return dumpTemporal(argv[2], argv[3]);
	}
	if (argc >= 4 && std::strcmp(argv[1], "sobol") == 0) {
		return dumpSobol(argv[2], argv[3]);
	}
	if (argc >= 4 && std::strcmp(argv[1], "upsample") == 0) {
		return dumpUpsample(argv[2], argv[3]);
	}
	if (argc >= 4 && std::strcmp(argv[1], "upscale") == 0) {
		return dumpUpscale(argv[2], argv[3]);
	}
	if (argc >= 5 && std::strcmp(argv[1], "bsdf") == 0) {
		return dumpBsdf(argv[2], argv[3], argv[4]);
	}
	if (argc >= 4 && std::strcmp(argv[1], "denoise") == 0) {
		return dumpDenoise(argv[2], argv[3]);
	}
	if (argc >= 4 && std::strcmp(argv[1], "scene") == 0) {
		return dumpScene(argv[2], argv[3]);
	}
	if (argc >= 5 && std::strcmp(argv[1], "trace") == 0) {
		return dumpTrace(argv[2], argv[3], argv[4]);
	}
	if (argc >= 5 && std::strcmp(argv[1], "cut") == 0) {
		return dumpCut(argv[2], std::atoi(argv[3]), argv[4]);
	}
	if (argc >= 5 && std::strcmp(argv[1], "cells") == 0) {
		return dumpCells(argv[2], argv[3], argv[4]);
	}
	std::fprintf(stderr, "usage: kdn_ref_dump scene|trace|cut|cells|bsdf|denoise|temporal|upscale|upsample|sobol ...\n");
	return 2;
}
