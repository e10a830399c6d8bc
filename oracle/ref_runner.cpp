// ref_runner - drives the reference's own enumeration kernels on a GPU.
//
// TEST INFRASTRUCTURE ONLY (the oracle's pin, never part of the product).
//
//   ref_runner <cumbe_ref.cubin> <graph.bi> [cuMBE|noRS|noES|noWS] [device|managed]
//
// The cubin holds the reference's kernels compiled from its unmodified
// sources (oracle/build_ref.py).  This program restates the reference's
// host driver (NTUDDSNLab/cuMBE src/main.cu:9-234) with the CUDA driver
// API: parse the .bi file (:38-48), size the grid from occupancy (:50-63),
// swap sides when rows > cols (:65-70), initialise the template state
// (:72-86) and the per-block state (:88-110), launch CUDA_GLOBAL_EXTENSION
// and CUDA_TRANSPOSE cooperatively (:143-146), order the roots by degree
// (src/header.cuh:55-63 via :147), launch CUDA_MBE_<variant> cooperatively
// (:190-199) and print the reference's own output lines (:207, :223).
//
// Differences, none of which changes what the kernels compute:
//  - plain device memory instead of managed memory, unless the fifth
//    argument is "managed" (then every buffer is managed memory, allocated
//    with cuMemAllocManaged as src/main.cu allocates with cudaMallocManaged,
//    and cleared as the operating system clears new pages);
//  - CUDA_TRANSPOSE's two `long long*` size arguments get 8-byte buffers
//    holding the sizes (the reference passes 4-byte ints there and relies
//    on zero padding, src/main.cu:112-113 vs src/transpose.cuh:1);
//  - every per-block array has one spare block of padding at its end, so
//    an index one past a block's slice never leaves the allocation.
#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#define CK(x)                                                                            \
    do {                                                                                 \
        CUresult r__ = (x);                                                              \
        if (r__ != CUDA_SUCCESS) {                                                       \
            const char* s__ = nullptr;                                                   \
            cuGetErrorString(r__, &s__);                                                 \
            std::fprintf(stderr, "ref_runner: %s failed: %s\n", #x, s__ ? s__ : "?");     \
            std::exit(3);                                                                \
        }                                                                                \
    } while (0)

struct Node {
    int start, length;
};

static bool g_managed = false;

static CUdeviceptr dalloc(size_t bytes) {
    CUdeviceptr p;
    if (g_managed)
        CK(cuMemAllocManaged(&p, bytes ? bytes : 8, CU_MEM_ATTACH_GLOBAL));
    else
        CK(cuMemAlloc(&p, bytes ? bytes : 8));
    CK(cuMemsetD8(p, 0, bytes ? bytes : 8));
    return p;
}

template <typename T>
static CUdeviceptr dcopy(const std::vector<T>& v, size_t extra_elems = 0) {
    CUdeviceptr p = dalloc(sizeof(T) * (v.size() + extra_elems));
    if (!v.empty()) CK(cuMemcpyHtoD(p, v.data(), sizeof(T) * v.size()));
    return p;
}

static CUfunction find(CUmodule mod, const char* needle) {
    unsigned int n = 0;
    CK(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> fs(n);
    CK(cuModuleEnumerateFunctions(fs.data(), n, mod));
    for (CUfunction f : fs) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        // mangled names embed the identifier length: "<len><name>" then params
        std::string want = std::to_string(std::strlen(needle)) + needle;
        if (name && std::strstr(name, want.c_str())) return f;
    }
    std::fprintf(stderr, "ref_runner: kernel %s not found in the cubin\n", needle);
    std::exit(3);
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <cubin> <graph.bi> [cuMBE|noRS|noES|noWS]\n", argv[0]);
        return 2;
    }
    std::string algo = argc > 3 ? argv[3] : "cuMBE";
    g_managed = argc > 4 && std::string(argv[4]) == "managed";
    algo = (algo == "noRS" || algo == "noES" || algo == "noWS") ? algo : "cuMBE";

    // .bi reader (src/main.cu:38-48)
    std::ifstream fin(argv[2]);
    if (!fin) {
        std::fprintf(stderr, "ref_runner: cannot open %s\n", argv[2]);
        return 2;
    }
    int NUM_R = 0, NUM_L = 0, NUM_EDGES = 0, ignored;
    fin >> NUM_R >> NUM_L >> NUM_EDGES;
    std::vector<Node> node_r_h(NUM_R), node_l_h(NUM_L);
    std::vector<int> edge_r_h(NUM_EDGES), edge_l_h(NUM_EDGES, 0);
    for (int i = 0; i < NUM_R; i++) fin >> node_r_h[i].start >> node_r_h[i].length;
    for (int i = 0; i < NUM_EDGES; i++) fin >> edge_r_h[i] >> ignored;
    if (!fin) {
        std::fprintf(stderr, "ref_runner: malformed .bi file\n");
        return 2;
    }

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[1]));
    CUfunction k_ext = find(mod, "CUDA_GLOBAL_EXTENSION");
    CUfunction k_tr = find(mod, "CUDA_TRANSPOSE");
    CUfunction k_mbe = find(mod, ("CUDA_MBE_" + algo).c_str());
    CUfunction k_occ = find(mod, "CUDA_MBE_cuMBE");

    // launch geometry (src/main.cu:50-63): 512 threads, grid = min(999, SMs x occupancy)
    const int numThreads = 512;
    int sms = 0, perSM = 0;
    CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
    CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_occ, numThreads, 0));
    int numBlocks_max = sms * perSM;
    int numBlocks = 999 > numBlocks_max ? numBlocks_max : 999;
    if (numBlocks < 1) numBlocks = 1;

    // device CSR in file orientation, then the swap (src/main.cu:65-70)
    CUdeviceptr node_r = dcopy(node_r_h), edge_r = dcopy(edge_r_h);
    CUdeviceptr node_l = dcopy(node_l_h), edge_l = dcopy(edge_l_h);
    bool swap_RL = NUM_R > NUM_L;
    if (swap_RL) {
        std::swap(NUM_L, NUM_R);
        std::swap(node_l, node_r);
        std::swap(edge_l, edge_r);
    }
    const size_t L = (size_t)NUM_L, R = (size_t)NUM_R, B = (size_t)numBlocks;

    // template state (src/main.cu:72-86)
    auto order = [](size_t n) {
        std::vector<int> v(n);
        for (size_t i = 0; i < n; i++) v[i] = (int)i;
        return v;
    };
    auto fill = [](size_t n, int val) { return std::vector<int>(n, val); };
    CUdeviceptr u2L = dcopy(order(L)), v2P = dcopy(order(R)), v2Q = dcopy(order(R));
    CUdeviceptr Lt = dcopy(order(L)), Rt = dcopy(order(R)), Pt = dcopy(order(R)), Qt = dcopy(order(R));
    CUdeviceptr xt = dcopy(fill(R, -1)), L_lp = dcopy(fill(R, NUM_L)), R_lp = dcopy(fill(R, 0));
    CUdeviceptr P_lp = dcopy(fill(R, NUM_R)), Q_lp = dcopy(fill(R, 0)), L_buf = dcopy(fill(L, 0));
    CUdeviceptr num_N_u = dcopy(fill(R, 0)), pre_min = dcopy(fill(R, 1));

    // per-block state (src/main.cu:88-110), one spare block of padding each
    auto per_block = [&](size_t n) { return dalloc(sizeof(int) * n * (B + 1)); };
    CUdeviceptr g_u2L = per_block(L), g_v2P = per_block(R), g_v2Q = per_block(R), g_L = per_block(L),
                g_R = per_block(R), g_P = per_block(R), g_Q = per_block(R), g_x = per_block(R),
                g_L_lp = per_block(R), g_R_lp = per_block(R), g_P_lp = per_block(R), g_Q_lp = per_block(R),
                g_L_buf = per_block(L), g_num_N_u = per_block(R), g_pre_min = per_block(R);
    CUdeviceptr ori_P = dalloc(sizeof(int) * (R + 1)), ori_P1 = per_block(R), ori_Q1 = per_block(R),
                ori_L1 = per_block(L);
    CUdeviceptr P_ptr1 = dalloc(sizeof(int) * (B + 1)), fix_P_ptr1 = dalloc(sizeof(int) * (B + 1)),
                fix_Q_ptr1 = dalloc(sizeof(int) * (B + 1));
    CUdeviceptr num_mb = dalloc(sizeof(int)), time_section = dalloc(sizeof(long long) * 11);
    CUdeviceptr tmp = dalloc(sizeof(int) * (std::max(L, R) + 1));
    CUdeviceptr dNUM_L = dcopy(std::vector<int>{NUM_L}), dNUM_R = dcopy(std::vector<int>{NUM_R}),
                dNUM_E = dcopy(std::vector<int>{NUM_EDGES});
    CUdeviceptr dNUM_L64 = dcopy(std::vector<long long>{NUM_L}), dNUM_R64 = dcopy(std::vector<long long>{NUM_R});

    // CUDA_GLOBAL_EXTENSION (src/main.cu:114-116,143)
    void* args_ext[] = {&g_u2L, &g_v2P, &g_v2Q, &g_L, &g_R, &g_P, &g_Q, &g_x, &g_L_lp, &g_R_lp, &g_P_lp, &g_Q_lp,
                        &g_L_buf, &g_num_N_u, &g_pre_min, &u2L, &v2P, &v2Q, &Lt, &Rt, &Pt, &Qt, &xt, &L_lp,
                        &R_lp, &P_lp, &Q_lp, &L_buf, &num_N_u, &pre_min, &dNUM_L, &dNUM_R};
    CK(cuLaunchCooperativeKernel(k_ext, numBlocks, 1, 1, numThreads, 1, 1, 0, nullptr, args_ext));
    CK(cuCtxSynchronize());
    // CUDA_TRANSPOSE (src/main.cu:112-113,145)
    void* args_csr2csc[] = {&dNUM_R64, &dNUM_L64, &dNUM_E, &node_r, &edge_r, &node_l, &edge_l, &tmp};
    void* args_csc2csr[] = {&dNUM_L64, &dNUM_R64, &dNUM_E, &node_l, &edge_l, &node_r, &edge_r, &tmp};
    CK(cuLaunchCooperativeKernel(k_tr, numBlocks, 1, 1, numThreads, 1, 1, 0, nullptr,
                                 swap_RL ? args_csc2csr : args_csr2csc));
    CK(cuCtxSynchronize());
    // root order: R ids by degree descending with std::sort (src/header.cuh:55-63)
    std::vector<Node> nr(R);
    if (R) CK(cuMemcpyDtoH(nr.data(), node_r, sizeof(Node) * R));
    std::vector<std::pair<int, int>> res;
    for (size_t i = 0; i < R; i++) res.push_back({(int)i, nr[i].length});
    std::sort(res.begin(), res.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
        return a.second > b.second;
    });
    std::vector<int> ori(R);
    for (size_t i = 0; i < R; i++) ori[i] = res[i].first;
    if (R) CK(cuMemcpyHtoD(ori_P, ori.data(), sizeof(int) * R));

    // CUDA_MBE_<variant> (src/main.cu:117-119,190-204)
    void* args_mbe[] = {&dNUM_L, &dNUM_R, &dNUM_E, &node_l, &edge_l, &node_r, &edge_r, &g_u2L, &g_v2P, &g_v2Q,
                        &g_L, &g_R, &g_P, &g_Q, &g_x, &g_L_lp, &g_R_lp, &g_P_lp, &g_Q_lp, &g_L_buf, &g_num_N_u,
                        &g_pre_min, &ori_P, &ori_P1, &ori_Q1, &ori_L1, &P_ptr1, &fix_P_ptr1, &fix_Q_ptr1, &num_mb,
                        &time_section};
    CUevent e0, e1;
    CK(cuEventCreate(&e0, 0));
    CK(cuEventCreate(&e1, 0));
    CK(cuEventRecord(e0, nullptr));
    CK(cuLaunchCooperativeKernel(k_mbe, numBlocks, 1, 1, numThreads, 1, 1, 0, nullptr, args_mbe));
    CK(cuCtxSynchronize());
    CK(cuEventRecord(e1, nullptr));
    CK(cuEventSynchronize(e1));
    float ms = 0;
    CK(cuEventElapsedTime(&ms, e0, e1));
    int count = 0;
    CK(cuMemcpyDtoH(&count, num_mb, sizeof(int)));
    std::printf("algorithm: %s\n|R|: %d, |L|: %d, |E|: %d\ngrid_size: %d, block_size: %d\n", algo.c_str(), NUM_R,
                NUM_L, NUM_EDGES, numBlocks, numThreads);
    std::printf("maximal bicliques: %d\nruntime (s): %g\nmemory: %s\n", count, ms / 1000.0,
                g_managed ? "managed" : "device");
    CK(cuModuleUnload(mod));
    CK(cuDevicePrimaryCtxRelease(dev));
    return 0;
}
