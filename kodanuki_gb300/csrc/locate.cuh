// Locating the octree leaf a point lies in (the trace kernel's descent),
// for the device and, to check it, the host.
#pragma once

#include "program.cuh"
#include "world.h"

namespace kdn {

// A read-only load: through the read-only data cache on the device.
template <typename T>
KDN_HD T loadOnce(const T* p) {
#ifdef __CUDA_ARCH__
	return __ldg(p);
#else
	return *p;
#endif
}

struct Located {
	uint32_t leaf;
	float lo[3], hi[3];
};

KDN_HD Located locate(const DeviceWorld& w, const float p[3]) {
	Located l;
	int32_t node;
	if (w.grid != nullptr) {
		// the grid cell: an estimate from the coordinates, set right against
		// the walls (the descent's own midpoints: a point on a wall goes up)
		const int n = 1 << w.gridLevel;
		int cell[3];
		for (int a = 0; a < 3; ++a) {
			const float* walls = w.gridWalls + a * (n + 1);
			int i              = int(fminf(fmaxf((p[a] - w.lower[a]) * w.gridScale[a], 0.0f), float(n - 1)));
			if (i > 0 && p[a] < loadOnce(walls + i)) --i;
			else if (i < n - 1 && p[a] >= loadOnce(walls + i + 1)) ++i;
			cell[a] = i;
		}
		const GridCell g = w.grid[(size_t(cell[2]) * n + cell[1]) * n + cell[0]];
		node             = g.node;
		// the box of the cell's level (a leaf above the grid's level is bigger)
		const int shift = int(w.gridLevel) - int(g.level);
		for (int a = 0; a < 3; ++a) {
			const float* walls = w.gridWalls + a * (n + 1);
			const int i0       = (cell[a] >> shift) << shift;
			l.lo[a]            = loadOnce(walls + i0);
			l.hi[a]            = loadOnce(walls + i0 + (1 << shift));
		}
	} else {
		for (int a = 0; a < 3; ++a) {
			l.lo[a] = w.lower[a];
			l.hi[a] = w.lower[a] + w.size[a];
		}
		node = loadOnce(&w.nodes[0]);
	}
	uint32_t at = 0;
	for (int depth = 0; depth < 30 && node >= 0; ++depth) {
		int o = 0;
		for (int a = 0; a < 3; ++a) {
			const float mid = 0.5f * (l.lo[a] + l.hi[a]);
			if (p[a] >= mid) {
				o |= 1 << a;
				l.lo[a] = mid;
			} else {
				l.hi[a] = mid;
			}
		}
		at   = uint32_t(node) + uint32_t(o);
		node = loadOnce(&w.nodes[at]);
	}
	l.leaf = uint32_t(~node);
	return l;
}

// The descent from the root alone, the reference for locate()'s grid.
KDN_HD uint32_t descendFromRoot(const DeviceWorld& w, const float p[3]) {
	float lo[3], hi[3];
	for (int a = 0; a < 3; ++a) {
		lo[a] = w.lower[a];
		hi[a] = w.lower[a] + w.size[a];
	}
	int32_t node = w.nodes[0];
	for (int depth = 0; depth < 30 && node >= 0; ++depth) {
		int o = 0;
		for (int a = 0; a < 3; ++a) {
			const float mid = 0.5f * (lo[a] + hi[a]);
			if (p[a] >= mid) {
				o |= 1 << a;
				lo[a] = mid;
			} else {
				hi[a] = mid;
			}
		}
		node = w.nodes[uint32_t(node) + uint32_t(o)];
	}
	return uint32_t(~node);
}

} // namespace kdn
