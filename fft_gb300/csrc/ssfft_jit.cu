// ssfft_jit.cu -- plan-time compilation of the size-specialised kernels in ssfft_codelets.cuh.
//
// Each plan names the template instantiations it needs (e.g.
// "ssfft_cl::batch<float, 1920, 128, 2, 2041, 1, false, false, 16, 16, 8, 3, 5>").  They are
// compiled once per process and device with NVRTC for the device's own architecture (sm_103a on
// GB300), loaded with the driver API and launched with cuLaunchKernel.  Compiled images are also
// kept on disk (SSFFT_CACHE_DIR, default ~/.cache/ssfft) keyed by a hash of the kernel source,
// the options and the instantiation names, so a second process skips the compile.
//
// The few driver-API calls are resolved through cudaGetDriverEntryPointByVersion rather than
// by linking libcuda, so the library also loads (for its host-only entry points) on a machine
// without a GPU driver.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

static const char *kCodeletSource =
#include "ssfft_codelets_src.inc"
    ;

namespace {

// Driver entry points (CUDA 12.0 ABI).
struct Driver {
	CUresult (*moduleLoadData)(CUmodule *, const void *) = nullptr;
	CUresult (*moduleUnload)(CUmodule) = nullptr;
	CUresult (*moduleGetFunction)(CUfunction *, CUmodule, const char *) = nullptr;
	CUresult (*funcSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
	CUresult (*funcGetAttribute)(int *, CUfunction_attribute, CUfunction) = nullptr;
	CUresult (*launchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
	                         void **, void **) = nullptr;
	CUresult (*getErrorString)(CUresult, const char **) = nullptr;
	CUresult (*occupancy)(int *, CUfunction, int, size_t) = nullptr;
	bool ok = false;
};

Driver g_drv;
std::once_flag g_drv_once;

template <typename F>
bool resolve(const char *sym, F &fn) {
	void *p = nullptr;
	cudaDriverEntryPointQueryResult q;
	if (cudaGetDriverEntryPointByVersion(sym, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
	    q != cudaDriverEntryPointSuccess || !p)
		return false;
	fn = reinterpret_cast<F>(p);
	return true;
}

const Driver &driver() {
	std::call_once(g_drv_once, [] {
		Driver d;
		d.ok = resolve("cuModuleLoadData", d.moduleLoadData) && resolve("cuModuleUnload", d.moduleUnload) &&
		       resolve("cuModuleGetFunction", d.moduleGetFunction) &&
		       resolve("cuFuncSetAttribute", d.funcSetAttribute) && resolve("cuFuncGetAttribute", d.funcGetAttribute) &&
		       resolve("cuLaunchKernel", d.launchKernel) &&
		       resolve("cuGetErrorString", d.getErrorString) &&
		       resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", d.occupancy);
		g_drv = d;
	});
	return g_drv;
}

struct Module {
	CUmodule mod = nullptr;
	std::vector<CUfunction> fns;
	long long smem_set = -1;  // dynamic shared memory the functions' attributes allow so far
};

std::mutex g_jit_mutex;
std::map<std::string, std::unique_ptr<Module>> g_modules;  // key: device + names
thread_local std::string g_jit_log;

uint64_t fnv1a(const std::string &s, uint64_t h = 1469598103934665603ull) {
	for (unsigned char ch : s) {
		h ^= ch;
		h *= 1099511628211ull;
	}
	return h;
}

std::string cache_dir() {
	const char *env = std::getenv("SSFFT_CACHE_DIR");
	std::string d;
	if (env && *env) {
		d = env;
	} else {
		const char *home = std::getenv("HOME");
		d = std::string(home && *home ? home : "/tmp") + "/.cache/ssfft";
	}
	return d;
}

void mkdirs(const std::string &path) {
	std::string cur;
	std::stringstream ss(path);
	std::string part;
	if (!path.empty() && path[0] == '/') cur = "/";
	while (std::getline(ss, part, '/')) {
		if (part.empty()) continue;
		cur += part + "/";
		mkdir(cur.c_str(), 0755);
	}
}

bool read_file(const std::string &path, std::string &out) {
	std::ifstream f(path, std::ios::binary);
	if (!f) return false;
	std::stringstream ss;
	ss << f.rdbuf();
	out = ss.str();
	return true;
}

void write_file_atomic(const std::string &path, const std::string &data) {
	const std::string tmp = path + ".tmp" + std::to_string(getpid());
	{
		std::ofstream f(tmp, std::ios::binary);
		if (!f) return;
		f.write(data.data(), (std::streamsize)data.size());
		if (!f) return;
	}
	std::rename(tmp.c_str(), path.c_str());
}

ssfft_status nvrtc_fail(nvrtcResult r, const char *what, const std::string &log) {
	g_jit_log = std::string(what) + ": " + nvrtcGetErrorString(r) + "\n" + log;
	return SSFFT_ERR_CUDA;
}

ssfft_status cu_fail(CUresult r, const char *what) {
	const char *s = nullptr;
	if (driver().getErrorString) driver().getErrorString(r, &s);
	g_jit_log = std::string(what) + ": " + (s ? s : "unknown driver error");
	return r == CUDA_ERROR_OUT_OF_MEMORY ? SSFFT_ERR_ALLOC : SSFFT_ERR_CUDA;
}

// Compile `names` to a cubin for `arch`, returning the image and the lowered names.
ssfft_status compile(const std::vector<std::string> &names, const std::string &arch, std::string &image,
                     std::vector<std::string> &lowered) {
	nvrtcProgram prog;
	nvrtcResult r = nvrtcCreateProgram(&prog, kCodeletSource, "ssfft_codelets.cu", 0, nullptr, nullptr);
	if (r != NVRTC_SUCCESS) return nvrtc_fail(r, "nvrtcCreateProgram", "");
	for (const auto &n : names) nvrtcAddNameExpression(prog, n.c_str());
	const std::string archopt = "--gpu-architecture=" + arch;
	std::vector<const char *> opts = {archopt.c_str(), "-std=c++17", "-lineinfo"};
	const bool verbose = debug_knob("jit_verbose", 0) != 0;
	if (verbose) opts.push_back("--ptxas-options=-v");
	r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
	size_t log_size = 0;
	nvrtcGetProgramLogSize(prog, &log_size);
	std::string log(log_size, '\0');
	if (log_size) nvrtcGetProgramLog(prog, &log[0]);
	if (verbose) std::fprintf(stderr, "[ssfft jit] %s\n%s\n", names.empty() ? "" : names[0].c_str(), log.c_str());
	if (r != NVRTC_SUCCESS) {
		nvrtcDestroyProgram(&prog);
		return nvrtc_fail(r, "nvrtcCompileProgram", log);
	}
	size_t sz = 0;
	r = nvrtcGetCUBINSize(prog, &sz);
	if (r != NVRTC_SUCCESS || sz == 0) {
		nvrtcDestroyProgram(&prog);
		return nvrtc_fail(r, "nvrtcGetCUBINSize", log);
	}
	image.resize(sz);
	nvrtcGetCUBIN(prog, &image[0]);
	lowered.clear();
	for (const auto &n : names) {
		const char *low = nullptr;
		r = nvrtcGetLoweredName(prog, n.c_str(), &low);
		if (r != NVRTC_SUCCESS || !low) {
			nvrtcDestroyProgram(&prog);
			return nvrtc_fail(r, "nvrtcGetLoweredName", n);
		}
		lowered.push_back(low);
	}
	nvrtcDestroyProgram(&prog);
	return SSFFT_SUCCESS;
}

}  // namespace

const char *jit_last_log() { return g_jit_log.c_str(); }

std::string device_arch(int device) {
	int major = 0, minor = 0;
	cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
	cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
	char buf[32];
	// arch-specific ("a") targets on Hopper and later expose the full instruction set
	std::snprintf(buf, sizeof buf, "sm_%d%d%s", major, minor, major >= 9 ? "a" : "");
	return buf;
}

// Compile (or fetch) the kernels `names` for the current device.  On success fns[i] is the
// kernel for names[i], with its dynamic shared-memory limit raised to `smem_bytes`.
ssfft_status jit_kernels(const std::vector<std::string> &names, size_t smem_bytes, std::vector<CUfunction> &fns) {
	int device = 0;
	cudaError_t ce = cudaGetDevice(&device);
	if (ce != cudaSuccess) return cuda_fail(ce, "cudaGetDevice");
	const Driver &drv = driver();
	if (!drv.ok) {
		g_jit_log = "CUDA driver entry points unavailable";
		return SSFFT_ERR_CUDA;
	}
	const std::string arch = device_arch(device);
	std::string key = std::to_string(device) + "|" + arch;
	Module *mod = nullptr;
	for (const auto &n : names) key += "|" + n;

	{
		std::lock_guard<std::mutex> lock(g_jit_mutex);
		auto it = g_modules.find(key);
		if (it != g_modules.end()) {
			fns = it->second->fns;
			mod = it->second.get();
			goto loaded;
		}
	}
	{
		// compile (or read from disk) without holding the lock, so plans compile concurrently
		const uint64_t h = fnv1a(key.substr(key.find('|') + 1), fnv1a(kCodeletSource));
		char hbuf[32];
		std::snprintf(hbuf, sizeof hbuf, "%016llx", (unsigned long long)h);
		const std::string dir = cache_dir();
		const std::string img_path = dir + "/" + hbuf + ".cubin", names_path = dir + "/" + hbuf + ".names";
		std::string image, names_txt;
		std::vector<std::string> lowered;
		bool cached = read_file(img_path, image) && read_file(names_path, names_txt);
		if (cached) {
			std::stringstream ss(names_txt);
			std::string line;
			while (std::getline(ss, line))
				if (!line.empty()) lowered.push_back(line);
			cached = lowered.size() == names.size() && !image.empty();
		}
		if (!cached) {
			ssfft_status st = compile(names, arch, image, lowered);
			if (st != SSFFT_SUCCESS) return st;
			mkdirs(dir);
			std::string txt;
			for (const auto &l : lowered) txt += l + "\n";
			write_file_atomic(img_path, image);
			write_file_atomic(names_path, txt);
		}
		ce = cudaFree(nullptr);  // make the runtime's primary context current for the driver calls
		if (ce != cudaSuccess) return cuda_fail(ce, "cudaFree(0)");
		std::lock_guard<std::mutex> lock(g_jit_mutex);
		auto it = g_modules.find(key);
		if (it == g_modules.end()) {
			std::unique_ptr<Module> m(new Module());
			CUresult r = drv.moduleLoadData(&m->mod, image.data());
			if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleLoadData");
			for (const auto &l : lowered) {
				CUfunction f = nullptr;
				r = drv.moduleGetFunction(&f, m->mod, l.c_str());
				if (r != CUDA_SUCCESS) {
					drv.moduleUnload(m->mod);
					return cu_fail(r, "cuModuleGetFunction");
				}
				m->fns.push_back(f);
			}
			it = g_modules.emplace(key, std::move(m)).first;
		}
		fns = it->second->fns;
		mod = it->second.get();
	}
loaded: {
	// attributes only when they change: a cached module needs no driver call at all, so plans
	// can be launched inside a stream capture
	std::lock_guard<std::mutex> lock(g_jit_mutex);
	if ((long long)smem_bytes > mod->smem_set) {
		for (CUfunction f : fns) {
			CUresult r = drv.funcSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem_bytes);
			if (r != CUDA_SUCCESS) return cu_fail(r, "cuFuncSetAttribute");
			// prefer the largest shared-memory carveout so smem, not the L1 split, bounds occupancy
			r = drv.funcSetAttribute(f, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100);
			if (r != CUDA_SUCCESS) return cu_fail(r, "cuFuncSetAttribute(carveout)");
		}
		mod->smem_set = (long long)smem_bytes;
	}
}
	return SSFFT_SUCCESS;
}

// Compile without loading (no GPU needed): checks that `names` build for `arch`.
ssfft_status jit_compile_only(const std::vector<std::string> &names, const std::string &arch, size_t *image_bytes) {
	std::string image;
	std::vector<std::string> lowered;
	ssfft_status st = compile(names, arch, image, lowered);
	if (image_bytes) *image_bytes = image.size();
	return st;
}

ssfft_status jit_launch_grid(CUfunction f, unsigned grid_x, unsigned grid_y, unsigned block, size_t smem,
                             cudaStream_t stream, void *args) {
	void *params[] = {args};
	CUresult r =
	    driver().launchKernel(f, grid_x, grid_y, 1, block, 1, 1, (unsigned)smem, (CUstream)stream, params, nullptr);
	if (r != CUDA_SUCCESS) return cu_fail(r, "cuLaunchKernel");
	return SSFFT_SUCCESS;
}

int jit_occupancy(CUfunction f, int block, size_t smem) {
	int n = 0;
	if (!driver().occupancy || driver().occupancy(&n, f, block, smem) != CUDA_SUCCESS) return 1;
	return n > 0 ? n : 1;
}

ssfft_status jit_launch(CUfunction f, unsigned grid, unsigned block, size_t smem, cudaStream_t stream, void *args) {
	return jit_launch_grid(f, grid, 1, block, smem, stream, args);
}

int jit_local_bytes(CUfunction f) {
	int n = 0;
	if (!driver().funcGetAttribute || driver().funcGetAttribute(&n, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, f) != CUDA_SUCCESS)
		return 0;
	return n;
}

std::string jit_cache_dir() { return cache_dir(); }
uint64_t codelet_hash() { return fnv1a(kCodeletSource); }
bool cache_read(const std::string &path, std::string &out) { return read_file(path, out); }
void cache_write(const std::string &path, const std::string &data) {
	mkdirs(cache_dir());
	write_file_atomic(path, data);
}

}  // namespace ssfft
