// tests/emu/emu_queue_main.cpp -- runs one emulated launch of an uneven-batch queue kernel
// (ssfft_cl::queue).  Compiled together with a generated case table (emu_queue_cases.inc:
// `{&ssfft_cl::queue<...>, cta_threads, smem_bytes, scalar_bytes},` lines).
// argv: case index, member-index file (int32 per item), thread-offset file (int32 per item and
//       thread), members file (int64 per member: n, tw offset, roots offset, threads per
//       transform; offsets in elements of the tables file), tables file (the kernel's dtype),
//       input file, output file (pre-filled; rewritten), prefetch distance (items ahead).
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
}

struct QCase {
	void (*fn)(const ssfft_cl::QueueArgs);
	int cta_threads;
	size_t smem;
	size_t scalar_bytes;
};
static const QCase kCases[] = {
#include "emu_queue_cases.inc"
};

static std::vector<char> slurp(const char *path) {
	std::ifstream f(path, std::ios::binary);
	return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

int main(int argc, char **argv) {
	if (argc != 9) return 2;
	const QCase &c = kCases[std::atoi(argv[1])];
	std::vector<char> kidx = slurp(argv[2]), toff = slurp(argv[3]), members = slurp(argv[4]), tab = slurp(argv[5]),
	                  in = slurp(argv[6]), out = slurp(argv[7]);
	const long long *mem = reinterpret_cast<const long long *>(members.data());
	const size_t nm = members.size() / (4 * sizeof(long long));
	std::vector<ssfft_cl::QSched> sch(nm);
	for (size_t k = 0; k < nm; ++k) {
		sch[k].n = mem[4 * k];
		sch[k].tw = tab.data() + mem[4 * k + 1] * c.scalar_bytes;
		sch[k].roots = tab.data() + mem[4 * k + 2] * c.scalar_bytes;
		sch[k].threads = mem[4 * k + 3];
	}
	ssfft_cl::QueueArgs a{};
	a.in = in.data();
	a.out = out.data();
	a.kidx = reinterpret_cast<const int *>(kidx.data());
	a.toff = reinterpret_cast<const int *>(toff.data());
	a.nitems = (long long)(kidx.size() / sizeof(int));
	if (toff.size() != (size_t)a.nitems * (size_t)c.cta_threads * sizeof(int)) return 6;
	a.sch = sch.data();
	a.pf_dist = std::atoll(argv[8]);
	if (c.smem > sizeof(ssfft_cl::smem_raw)) return 5;
	for (long long b = 0; b < a.nitems; ++b) {
		std::barrier<> bar(c.cta_threads);
		std::vector<std::thread> th;
		th.reserve(c.cta_threads);
		for (int t = 0; t < c.cta_threads; ++t)
			th.emplace_back([&, t, b] {
				threadIdx.x = (unsigned)t;
				blockIdx.x = (unsigned)b;
				gridDim.x = (unsigned)a.nitems;
				emu_barrier = &bar;
				c.fn(a);
			});
		for (auto &x : th) x.join();
	}
	std::ofstream f(argv[7], std::ios::binary);
	f.write(out.data(), (std::streamsize)out.size());
	return 0;
}
