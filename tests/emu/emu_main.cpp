// tests/emu/emu_main.cpp -- runs one emulated kernel launch.  Compiled together with a generated
// case table (emu_cases.inc: `{name, &ssfft_cl::batch<...>, cta_threads, smem_bytes[, cluster]},`
// lines).  Cluster kernels (cluster = 2) run their two CTAs at once, each with its own
// shared-memory array; reads of a CTA's shared memory through the cluster window are
// bounds-checked.
// argv: case index, grid, raw input file, raw output file (pre-filled), table file, batch,
//       in_dist, out_dist (scalars), scalar bytes, input bytes per transform (staged kernels)
//       [, offset-table file: int64 scalar offsets of each transform in input and output].
// The table file holds tw, roots, rtw, rot back to back in the kernel's dtype, preceded by four
// uint64 element counts (scalars).
#include "cuda_emu.h"
#include "ssfft_codelets.cuh"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <thread>
#include <vector>

thread_local EmuIdx threadIdx, blockIdx, gridDim;
thread_local std::barrier<> *emu_barrier;
std::atomic<int> emu_or_acc{0};
static size_t emu_smem_bytes = 0;
namespace ssfft_cl {
alignas(1024) unsigned char smem_raw[232 * 1024];
thread_local unsigned char *emu_cta_smem = nullptr, *emu_peer_smem = nullptr;
thread_local std::barrier<> *emu_cluster_barrier = nullptr;
float2 emu_cluster_load(ClusterSmem s, int i) {
	const unsigned char *p = reinterpret_cast<const unsigned char *>(s.base + i);
	const bool own = p >= emu_cta_smem && p + sizeof(float2) <= emu_cta_smem + emu_smem_bytes;
	const bool peer = p >= emu_peer_smem && p + sizeof(float2) <= emu_peer_smem + emu_smem_bytes;
	if (i < 0 || !(own || peer)) {
		std::fprintf(stderr, "cluster shared-memory read out of bounds: index %d\n", i);
		std::abort();
	}
	return s.base[i];
}
float emu_tmem[128][32];
// BF16 round to nearest even (finite inputs) and widening
unsigned short f2bf(float x) {
	uint32_t b;
	std::memcpy(&b, &x, 4);
	b += 0x7FFFu + ((b >> 16) & 1u);
	return (unsigned short)(b >> 16);
}
float bf2f(unsigned short h) {
	const uint32_t b = (uint32_t)h << 16;
	float x;
	std::memcpy(&x, &b, 4);
	return x;
}
}

struct Case {
	const char *name;
	void (*fn)(const ssfft_cl::Args);
	int cta_threads;
	size_t smem;
	int cluster;  // 0 / 1: one CTA at a time; 2: two CTAs of a cluster at once
};
static const Case kCases[] = {
#include "emu_cases.inc"
};

static std::vector<char> slurp(const char *path) {
	std::ifstream f(path, std::ios::binary);
	return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

int main(int argc, char **argv) {
	if (argc != 11 && argc != 12) return 2;
	const Case &c = kCases[std::atoi(argv[1])];
	const int grid = std::atoi(argv[2]);
	std::vector<char> in = slurp(argv[3]), out = slurp(argv[4]), tab = slurp(argv[5]);
	const size_t sb = (size_t)std::atoi(argv[9]);
	const uint64_t *cnt = reinterpret_cast<const uint64_t *>(tab.data());
	const char *base = tab.data() + 4 * sizeof(uint64_t);
	ssfft_cl::Args a{};
	a.in = in.data();
	a.out = out.data();
	a.batch = std::atoll(argv[6]);
	a.in_dist = std::atoll(argv[7]);
	a.out_dist = std::atoll(argv[8]);
	a.tw = base;
	a.roots = base + cnt[0] * sb;
	a.rtw = base + (cnt[0] + cnt[1]) * sb;
	a.rot = base + (cnt[0] + cnt[1] + cnt[2]) * sb;
	unsigned err = 0;
	a.err = &err;
	a.spin_limit = 1;
	a.in_bytes = (unsigned)std::atoi(argv[10]);
	std::vector<char> offs;
	if (argc == 12) {
		offs = slurp(argv[11]);
		a.offs = reinterpret_cast<const long long *>(offs.data());
	}
	// tensor-core kernels: the first pass's DFT matrix follows the four tables when present
	a.tcb = reinterpret_cast<const float *>(base + (cnt[0] + cnt[1] + cnt[2] + cnt[3]) * sb);
	if (c.cluster == 2) {
		emu_smem_bytes = c.smem;
		for (int b = 0; b + 1 < grid; b += 2) {
			// guard bytes around each CTA's array, checked afterwards (writes out of bounds)
			constexpr size_t kGuard = 4096;
			std::vector<unsigned char> sm[2] = {std::vector<unsigned char>(c.smem + 2 * kGuard, 0xA5),
			                                    std::vector<unsigned char>(c.smem + 2 * kGuard, 0xA5)};
			std::barrier<> cbar(2 * c.cta_threads), bar0(c.cta_threads), bar1(c.cta_threads);
			std::vector<std::thread> th;
			for (int q = 0; q < 2; ++q)
				for (int t = 0; t < c.cta_threads; ++t)
					th.emplace_back([&, t, q] {
						threadIdx.x = (unsigned)t;
						blockIdx.x = (unsigned)(b + q);
						gridDim.x = (unsigned)grid;
						emu_barrier = q ? &bar1 : &bar0;
						ssfft_cl::emu_cluster_barrier = &cbar;
						ssfft_cl::emu_cta_smem = sm[q].data() + kGuard;
						ssfft_cl::emu_peer_smem = sm[1 - q].data() + kGuard;
						c.fn(a);
					});
			for (auto &x : th) x.join();
			for (int q = 0; q < 2; ++q)
				for (size_t i = 0; i < kGuard; ++i)
					if (sm[q][i] != 0xA5 || sm[q][kGuard + c.smem + i] != 0xA5) {
						std::fprintf(stderr, "shared-memory write outside the CTA's %zu bytes\n", c.smem);
						return 4;
					}
		}
		if (err) return 3;
		std::ofstream f(argv[4], std::ios::binary);
		f.write(out.data(), (std::streamsize)out.size());
		return 0;
	}
	for (int b = 0; b < grid; ++b) {
		std::barrier<> bar(c.cta_threads);
		std::vector<std::thread> th;
		th.reserve(c.cta_threads);
		for (int t = 0; t < c.cta_threads; ++t)
			th.emplace_back([&, t, b] {
				threadIdx.x = (unsigned)t;
				blockIdx.x = (unsigned)b;
				gridDim.x = (unsigned)grid;
				emu_barrier = &bar;
				c.fn(a);
			});
		for (auto &x : th) x.join();
	}
	if (err) return 3;
	std::ofstream f(argv[4], std::ios::binary);
	f.write(out.data(), (std::streamsize)out.size());
	return 0;
}
