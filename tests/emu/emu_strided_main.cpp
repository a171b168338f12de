// tests/emu/emu_strided_main.cpp -- runs one emulated launch of a multi-pass (four-step) pass
// kernel, ssfft_cl::strided, or of its RealFFT split kernel, ssfft_cl::real_split.  Compiled
// together with generated case tables (emu_strided_cases.inc: `{name, &ssfft_cl::strided<...>,
// cta_threads, smem_bytes},` lines; emu_split_cases.inc: `{name, &ssfft_cl::real_split<...>},`).
// Pass: argv = "p<case>", grid, raw input file, raw output file (pre-filled), table file (the
//       plan's table bytes), transforms (U2), complex points per transform (the u2 strides), then
//       U0, U1, is0, is1, in_es, os0, os1, out_es and the table byte offsets of the pass twiddles,
//       roots, inter-pass twiddles (lo, hi) and half-shift rotations.
// Split: argv = "s<case>", blocks per transform, raw source file (the inverse's bins), raw buffer
//       file (pre-filled; split in place / pre-twiddled output), table file, transforms, complex
//       points per transform, table byte offset of the split twiddles.
// Bluestein element-wise kernels (emu_blue_cases.inc): argv = "b<case>", blocks per transform,
//       transforms, raw input file, raw output file, raw work file (both written back), table
//       file, n, m, distance between transforms, table byte offsets of the chirp and of the
//       spectrum of b [, table byte offsets of the half-shift rotations applied to the input and
//       to the output, -1 for none].
// Odd-length pack / unpack (emu_pack_cases.inc): argv = "k<case>", blocks per transform, raw
//       source file, raw destination file (pre-filled; written back), transforms, real length n,
//       complex points per transform h.
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
namespace ssfft_cl {
alignas(1024) unsigned char smem_raw[232 * 1024];
float emu_tmem[128][32];
thread_local unsigned char *emu_cta_smem = nullptr, *emu_peer_smem = nullptr;
thread_local std::barrier<> *emu_cluster_barrier = nullptr;
float2 emu_cluster_load(ClusterSmem s, int i) { return s.base[i]; }
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
}  // namespace ssfft_cl

struct Case {
	const char *name;
	void (*fn)(const ssfft_cl::StridedArgs);
	int cta_threads;
	size_t smem;
};
static const Case kCases[] = {
#include "emu_strided_cases.inc"
};
struct SplitCase {
	const char *name;
	void (*fn)(const ssfft_cl::SplitArgs);
};
static const SplitCase kSplitCases[] = {
#include "emu_split_cases.inc"
	{nullptr, nullptr}};

struct BlueCase {
	const char *name;
	void (*fn)(const ssfft_cl::BlueArgs);
};
static const BlueCase kBlueCases[] = {
#include "emu_blue_cases.inc"
	{nullptr, nullptr}};

struct PackCase {
	const char *name;
	void (*fn)(const ssfft_cl::PackArgs);
};
static const PackCase kPackCases[] = {
#include "emu_pack_cases.inc"
	{nullptr, nullptr}};

// real_split and the Bluestein kernels: 256 threads per block (no barriers), blockIdx.y =
// transform
static int run_split(int argc, char **argv);
static int run_blue(int argc, char **argv);
static int run_pack(int argc, char **argv);

static std::vector<char> slurp(const char *path) {
	std::ifstream f(path, std::ios::binary);
	return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

int main(int argc, char **argv) {
	if (argc > 1 && argv[1][0] == 's') return run_split(argc, argv);
	if (argc > 1 && argv[1][0] == 'b') return run_blue(argc, argv);
	if (argc > 1 && argv[1][0] == 'k') return run_pack(argc, argv);
	if (argc != 21 || argv[1][0] != 'p') return 2;
	const Case &c = kCases[std::atoi(argv[1] + 1)];
	const int grid = std::atoi(argv[2]);
	std::vector<char> in = slurp(argv[3]), out = slurp(argv[4]), tab = slurp(argv[5]);
	auto ll = [&](int i) { return std::atoll(argv[i]); };
	if (c.smem > sizeof ssfft_cl::smem_raw) return 5;
	ssfft_cl::StridedArgs a{};
	a.in = in.data();
	a.out = out.data();
	a.U2 = ll(6);
	const long long n = ll(7);
	a.is2 = a.os2 = n;
	a.rot_in_stride2 = a.rot_out_stride2 = n;
	a.U0 = ll(8);
	a.U1 = ll(9);
	a.is0 = ll(10);
	a.is1 = ll(11);
	a.in_es = ll(12);
	a.os0 = ll(13);
	a.os1 = ll(14);
	a.out_es = ll(15);
	a.tw = tab.data() + ll(16);
	a.roots = tab.data() + ll(17);
	a.twlo = tab.data() + ll(18);
	a.twhi = tab.data() + ll(19);
	a.rot = tab.data() + ll(20);
	a.pf_dist = 0;
	// one thread per CUDA thread of a CTA, reused for every CTA in turn (the barrier at the end
	// of a block keeps the CTAs apart: they share the emulated shared memory)
	std::barrier<> bar(c.cta_threads);
	std::vector<std::thread> th;
	th.reserve(c.cta_threads);
	for (int t = 0; t < c.cta_threads; ++t)
		th.emplace_back([&, t] {
			threadIdx.x = (unsigned)t;
			gridDim.x = (unsigned)grid;
			emu_barrier = &bar;
			for (int b = 0; b < grid; ++b) {
				blockIdx.x = (unsigned)b;
				c.fn(a);
				bar.arrive_and_wait();
			}
		});
	for (auto &x : th) x.join();
	std::ofstream f(argv[4], std::ios::binary);
	f.write(out.data(), (std::streamsize)out.size());
	return 0;
}

static int run_split(int argc, char **argv) {
	if (argc != 9) return 2;
	const SplitCase &c = kSplitCases[std::atoi(argv[1] + 1)];
	const int blocks = std::atoi(argv[2]);
	std::vector<char> src = slurp(argv[3]), buf = slurp(argv[4]), tab = slurp(argv[5]);
	ssfft_cl::SplitArgs a{};
	a.src = src.data();
	a.buf = buf.data();
	a.batch = std::atoll(argv[6]);
	a.dist = std::atoll(argv[7]);
	a.rtw = tab.data() + std::atoll(argv[8]);
	for (long long y = 0; y < a.batch; ++y)
		for (int b = 0; b < blocks; ++b)
			for (int t = 0; t < 256; ++t) {
				threadIdx.x = (unsigned)t;
				blockIdx.x = (unsigned)b;
				blockIdx.y = (unsigned)y;
				gridDim.x = (unsigned)blocks;
				c.fn(a);
			}
	std::ofstream f(argv[4], std::ios::binary);
	f.write(buf.data(), (std::streamsize)buf.size());
	return 0;
}

static int run_pack(int argc, char **argv) {
	if (argc != 8) return 2;
	const PackCase &c = kPackCases[std::atoi(argv[1] + 1)];
	const int blocks = std::atoi(argv[2]);
	std::vector<char> src = slurp(argv[3]), dst = slurp(argv[4]);
	ssfft_cl::PackArgs a{};
	a.src = src.data();
	a.dst = dst.data();
	a.batch = std::atoll(argv[5]);
	a.n = std::atoll(argv[6]);
	a.h = std::atoll(argv[7]);
	for (long long y = 0; y < a.batch; ++y)
		for (int b = 0; b < blocks; ++b)
			for (int t = 0; t < 256; ++t) {
				threadIdx.x = (unsigned)t;
				blockIdx.x = (unsigned)b;
				blockIdx.y = (unsigned)y;
				gridDim.x = (unsigned)blocks;
				c.fn(a);
			}
	std::ofstream f(argv[4], std::ios::binary);
	f.write(dst.data(), (std::streamsize)dst.size());
	return 0;
}

static int run_blue(int argc, char **argv) {
	if (argc != 13 && argc != 15) return 2;
	const BlueCase &c = kBlueCases[std::atoi(argv[1] + 1)];
	const int blocks = std::atoi(argv[2]);
	std::vector<char> in = slurp(argv[4]), out = slurp(argv[5]), work = slurp(argv[6]), tab = slurp(argv[7]);
	ssfft_cl::BlueArgs a{};
	a.in = in.data();
	a.out = out.data();
	a.work = work.data();
	a.batch = std::atoll(argv[3]);
	a.n = std::atoll(argv[8]);
	a.m = std::atoll(argv[9]);
	a.dist = std::atoll(argv[10]);
	a.chirp = tab.data() + std::atoll(argv[11]);
	a.bhat = tab.data() + std::atoll(argv[12]);
	if (argc == 15) {
		const long long ri = std::atoll(argv[13]), ro = std::atoll(argv[14]);
		a.rot_in = ri >= 0 ? tab.data() + ri : nullptr;
		a.rot_out = ro >= 0 ? tab.data() + ro : nullptr;
	}
	for (long long y = 0; y < a.batch; ++y)
		for (int b = 0; b < blocks; ++b)
			for (int t = 0; t < 256; ++t) {
				threadIdx.x = (unsigned)t;
				blockIdx.x = (unsigned)b;
				blockIdx.y = (unsigned)y;
				gridDim.x = (unsigned)blocks;
				c.fn(a);
			}
	std::ofstream fo(argv[5], std::ios::binary);
	fo.write(out.data(), (std::streamsize)out.size());
	std::ofstream fw(argv[6], std::ios::binary);
	fw.write(work.data(), (std::streamsize)work.size());
	return 0;
}
