// Test-oracle harness: the reference HashGrid's cell assignment
// (src/photon/hashgrid.cc, HashGrid::updateGrid) for given points.
// Input (binary): f64 cell_size, u32 grid_size, f32 box[6] (a xyz, g xyz),
//                 u32 n, f32 pos[n][3]
// Output (binary): u32 bucket[n]
// Only tests/golden/make_render_golden.py runs it.
#include "photon/hashgrid.h"
#include "photon/photon.h"
#include "geometry/bound.h"
#include <cstdio>
#include <vector>

int main(int argc, char **argv)
{
	if(argc != 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
	FILE *fi = fopen(argv[1], "rb");
	if(!fi) { perror("in"); return 2; }
	double cell;
	unsigned int grid_size, n;
	float box[6];
	if(fread(&cell, 8, 1, fi) != 1 || fread(&grid_size, 4, 1, fi) != 1 || fread(box, 4, 6, fi) != 6 || fread(&n, 4, 1, fi) != 1) return 2;
	std::vector<float> pos(3ull * n);
	if(fread(pos.data(), 4, pos.size(), fi) != pos.size()) return 2;
	fclose(fi);
	const yafaray::Point3f a{{box[0], box[1], box[2]}}, g{{box[3], box[4], box[5]}};
	yafaray::Bound<float> b{a, g};
	yafaray::HashGrid grid(cell, grid_size, b);
	for(unsigned int i = 0; i < n; ++i)
	{
		yafaray::Photon ph;
		ph.pos_ = yafaray::Point3f{{pos[3ull * i], pos[3ull * i + 1], pos[3ull * i + 2]}};
		grid.pushPhoton(std::move(ph));
	}
	grid.updateGrid();
	std::vector<unsigned int> bucket(n, 0xFFFFFFFFu);
	const yafaray::Photon *base = grid.photons_.data();
	for(unsigned int h = 0; h < grid_size; ++h)
		if(grid.hash_grid_[h])
			for(const yafaray::Photon *p : *grid.hash_grid_[h]) bucket[p - base] = h;
	FILE *fo = fopen(argv[2], "wb");
	if(!fo) { perror("out"); return 2; }
	fwrite(bucket.data(), 4, n, fo);
	fclose(fo);
	return 0;
}
