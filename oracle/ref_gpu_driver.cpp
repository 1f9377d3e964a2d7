/*
 * ref_gpu_driver.cpp -- runs the reference's OWN GPU kernels for key
 * generation, the active multi-search and the flush into the key-value +
 * bitmap store, as a second oracle for those stages.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/ and tests/golden/ scripts, never
 * by the product.  The kernels come from the reference's cuda/geometry.cu,
 * compiled unmodified for sm_103a into oracle/_ref/geometry.cubin by
 * oracle/build_ref.sh (a GPU binary: it is built where the reference sources
 * are and runs on any host of the GPU).  Their argument is the reference's
 * device-resident workbench; oracle/_ref/ref_gpu_layout.h (generated from the
 * reference's headers by oracle/ref_gpu_layout.cpp) gives the byte offsets
 * of the fields they use, and this file fills a workbench image the way
 * cuda_create_device_bench does (cuda/geometry.cu:1395-1565).
 *
 * Host-side steps of process_with_gpu's flush (cuda/geometry.cu:1752-2135)
 * are restated here: the thrust partition and sorts become host-side stable
 * partition and stable sorts (thrust's radix sorts are stable; the key sorts
 * have unique keys), and CTF::get_ctf_bits runs as the oracle's go_ctf_bits,
 * which tests/test_flush_oracle.py pins against the reference's own.  The
 * kernels themselves -- cuda_identify_meetings, set_oid, get_o_limit,
 * cuda_write_o_bitmap, narrow_xy_to_y, make_sid, write_sid_in_key,
 * get_CTF_capacity, cuda_get_limit, cuda_write_bitmap, write_key_and_mbr and
 * cuda_init_o_boxs -- are the reference's code, launched with the
 * reference's grid and block sizes in the reference's order.
 *
 * Callers must keep the inputs inside the reference's domain (the oracle
 * checks it first): the reference's kernels assert on keys without a CTF and
 * write bitmap bits wherever a box lands.  The bitmap array gets slack
 * beyond bitmaps_size so that bits the oracle reports as outside the array
 * stay in memory this driver owns.
 */
#include <cuda.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "glint_oracle.h"
#include "_ref/ref_gpu_layout.h"

typedef unsigned __int128 u128;

extern "C" {
typedef struct rg_config {
    uint32_t device, num_objects, CTF_count, split_num, min_meet_time, max_meet_time;
    uint64_t kv_capacity;
    double dProbFalse;
    double mbr[4];                 /* map box: low x, low y, high x, high y */
} rg_config;

typedef struct rg_flush_info {
    uint64_t kv_count, key_bytes;
    uint32_t oversize_kv_count, oversize_start_time_min, oversize_start_time_max, oversize_end_time_min,
        oversize_end_time_max, sid_count, oversize_oid_count, pad;
    uint64_t bits_in_slack;        /* bitmap bits the kernels set past the bitmap array */
} rg_flush_info;
}

namespace {

struct Kernels {
    CUfunction identify, init_o_boxs, set_oid, get_o_limit, write_o_bitmap, narrow_xy_to_y, make_sid,
        write_sid_in_key, get_ctf_capacity, get_limit, write_bitmap, write_key_and_mbr;
};

constexpr size_t kBitmapSlack = 4u << 20;

template <class T>
void put(std::vector<uint8_t> &img, size_t off, T v) {
    std::memcpy(img.data() + off, &v, sizeof(T));
}
template <class T>
T get(const std::vector<uint8_t> &img, size_t off) {
    T v;
    std::memcpy(&v, img.data() + off, sizeof(T));
    return v;
}

}  // namespace

struct rg_ctx {
    CUcontext ctx = nullptr;
    CUdevice dev = 0;
    CUmodule mod = nullptr;
    Kernels k{};
    uint32_t N = 0, CTF_count = 0, split_num = 0, max_meet_time = 0, min_meet_time = 0;
    uint64_t kv_capacity = 0;
    double mbr[4] = {0, 0, 0, 0};
    std::vector<uint8_t> wb, cfg;   /* host images of the workbench and its configuration */
    CUdeviceptr d_bench = 0, d_cfg = 0, d_keys = 0, d_ctf_keys = 0, d_kv_boxs = 0, d_mid_xys = 0, d_same = 0,
                d_sids = 0, d_o_boxs = 0, d_oids = 0, d_bitmaps = 0, d_capacity = 0, d_ctfs = 0;
    uint32_t bit_count = 0, bitmaps_size = 0;
    std::string err;
    /* last flush */
    rg_flush_info info{};
    std::vector<uint8_t> packed, bitmaps, o_bitmap;
    std::vector<uint16_t> sids;
    std::vector<uint32_t> capacity;
    std::vector<go_ctf_meta> ctfs;
    std::vector<u128> o_keys;
    std::vector<float> o_boxes;
};

namespace {

bool ok(rg_ctx *c, CUresult r, const char *what) {
    if (r == CUDA_SUCCESS) return true;
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    c->err = std::string(what) + ": " + (s ? s : "?");
    return false;
}

bool launch(rg_ctx *c, CUfunction f, uint64_t grid, unsigned block, const char *what, uint32_t *arg2 = nullptr) {
    void *args[2] = {&c->d_bench, arg2};
    if (!ok(c, cuLaunchKernel(f, (unsigned)grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr), what)) return false;
    return ok(c, cuCtxSynchronize(), what);
}

bool bench_down(rg_ctx *c) { return ok(c, cuMemcpyDtoH(c->wb.data(), c->d_bench, RG_WB_SIZE), "workbench to host"); }
bool bench_up(rg_ctx *c) {
    return ok(c, cuMemcpyHtoD(c->d_bench, c->wb.data(), RG_WB_SIZE), "workbench to device") &&
           ok(c, cuMemcpyHtoD(c->d_cfg, c->cfg.data(), RG_CFG_SIZE), "configuration to device");
}

bool alloc(rg_ctx *c, CUdeviceptr *p, size_t bytes) {
    return ok(c, cuMemAlloc(p, bytes ? bytes : 16), "cuMemAlloc") && ok(c, cuMemsetD8(*p, 0, bytes ? bytes : 16), "memset");
}

/* the state cuda_create_device_bench leaves, and the reset after each flush
 * (cuda/geometry.cu:2094-2113) */
bool reset_store(rg_ctx *c) {
    const size_t N = c->N;
    bool good = ok(c, cuMemsetD8(c->d_sids, 0, N * 2), "reset") && ok(c, cuMemsetD8(c->d_oids, 0, N * 4), "reset") &&
                ok(c, cuMemsetD8(c->d_bitmaps, 0, c->bitmaps_size + kBitmapSlack), "reset") &&
                ok(c, cuMemsetD8(c->d_same, 0, N * 4), "reset") && ok(c, cuMemsetD8(c->d_mid_xys, 0, N * 8), "reset") &&
                ok(c, cuMemsetD8(c->d_capacity, 0, c->CTF_count * 4), "reset") &&
                ok(c, cuMemsetD8(c->d_ctfs, 0, (size_t)c->CTF_count * RG_CTF_SIZE), "reset") &&
                ok(c, cuMemsetD8(c->d_ctf_keys, 0, c->kv_capacity * 16), "reset");
    if (!good || !bench_down(c)) return false;
    put<uint32_t>(c->wb, RG_WB_kv_count, 0);
    put<uint32_t>(c->wb, RG_WB_sid_count, 0);
    put<uint32_t>(c->wb, RG_WB_oversize_oid_count, 0);
    if (!bench_up(c)) return false;
    return launch(c, c->k.init_o_boxs, N / 1024 + 1, 1024, "cuda_init_o_boxs");
}

go_ctf_meta meta_of(const uint8_t *p) {
    go_ctf_meta m;
    std::memset(&m, 0, sizeof(m));
    std::memcpy(m.ctf_mbr, p + RG_CTF_ctf_mbr, 16);
    std::memcpy(&m.CTF_kv_capacity, p + RG_CTF_CTF_kv_capacity, 4);
    std::memcpy(&m.start_time_min, p + RG_CTF_start_time_min, 4);
    std::memcpy(&m.start_time_max, p + RG_CTF_start_time_max, 4);
    std::memcpy(&m.end_time_min, p + RG_CTF_end_time_min, 4);
    std::memcpy(&m.end_time_max, p + RG_CTF_end_time_max, 4);
    std::memcpy(&m.ctf_bitmap_size, p + RG_CTF_ctf_bitmap_size, 4);
    std::memcpy(&m.key_bit, p + RG_CTF_key_bit, 2);
    std::memcpy(&m.id_bit, p + RG_CTF_id_bit, 2);
    std::memcpy(&m.duration_bit, p + RG_CTF_duration_bit, 2);
    std::memcpy(&m.end_bit, p + RG_CTF_end_bit, 2);
    std::memcpy(&m.low_x_bit, p + RG_CTF_low_x_bit, 2);
    std::memcpy(&m.low_y_bit, p + RG_CTF_low_y_bit, 2);
    std::memcpy(&m.edge_bit, p + RG_CTF_edge_bit, 2);
    std::memcpy(&m.mbr_bit, p + RG_CTF_mbr_bit, 2);
    std::memcpy(&m.x_grid, p + RG_CTF_x_grid, 2);
    std::memcpy(&m.y_grid, p + RG_CTF_y_grid, 2);
    return m;
}

void meta_into(uint8_t *p, const go_ctf_meta &m) {
    std::memcpy(p + RG_CTF_ctf_bitmap_size, &m.ctf_bitmap_size, 4);
    std::memcpy(p + RG_CTF_key_bit, &m.key_bit, 2);
    std::memcpy(p + RG_CTF_id_bit, &m.id_bit, 2);
    std::memcpy(p + RG_CTF_duration_bit, &m.duration_bit, 2);
    std::memcpy(p + RG_CTF_end_bit, &m.end_bit, 2);
    std::memcpy(p + RG_CTF_low_x_bit, &m.low_x_bit, 2);
    std::memcpy(p + RG_CTF_low_y_bit, &m.low_y_bit, 2);
    std::memcpy(p + RG_CTF_edge_bit, &m.edge_bit, 2);
    std::memcpy(p + RG_CTF_mbr_bit, &m.mbr_bit, 2);
    std::memcpy(p + RG_CTF_x_grid, &m.x_grid, 2);
    std::memcpy(p + RG_CTF_y_grid, &m.y_grid, 2);
}

/* stable sort of n 8- or 16-byte keys with their 16-byte values, in place on
 * the device (thrust::sort_by_key) */
template <class K>
bool sort_by_key(rg_ctx *c, CUdeviceptr keys, CUdeviceptr vals, size_t n, size_t val_bytes) {
    if (n == 0) return true;
    std::vector<K> k(n);
    std::vector<uint8_t> v(n * val_bytes), v2(n * val_bytes);
    if (!ok(c, cuMemcpyDtoH(k.data(), keys, n * sizeof(K)), "sort") ||
        !ok(c, cuMemcpyDtoH(v.data(), vals, n * val_bytes), "sort"))
        return false;
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return k[a] < k[b]; });
    std::vector<K> k2(n);
    for (size_t i = 0; i < n; ++i) {
        k2[i] = k[idx[i]];
        std::memcpy(&v2[i * val_bytes], &v[idx[i] * val_bytes], val_bytes);
    }
    return ok(c, cuMemcpyHtoD(keys, k2.data(), n * sizeof(K)), "sort") &&
           ok(c, cuMemcpyHtoD(vals, v2.data(), n * val_bytes), "sort");
}

}  // namespace

extern "C" {

int rg_open(const char *cubin, const rg_config *cfg, rg_ctx **out) {
    *out = nullptr;
    rg_ctx *c = new rg_ctx();
    c->N = cfg->num_objects;
    c->CTF_count = cfg->CTF_count;
    c->split_num = cfg->split_num;
    c->max_meet_time = cfg->max_meet_time;
    c->min_meet_time = cfg->min_meet_time;
    c->kv_capacity = cfg->kv_capacity;
    std::memcpy(c->mbr, cfg->mbr, sizeof(c->mbr));
    c->bit_count = RG_BITMAP_EDGE * RG_BITMAP_EDGE;               /* tracing/filter.cpp:72-73 */
    c->bitmaps_size = c->bit_count / 8 * c->CTF_count;
    c->wb.assign(RG_WB_SIZE, 0);
    c->cfg.assign(RG_CFG_SIZE, 0);
    bool good = ok(c, cuInit(0), "cuInit") && ok(c, cuDeviceGet(&c->dev, cfg->device), "cuDeviceGet") &&
                ok(c, cuDevicePrimaryCtxRetain(&c->ctx, c->dev), "primary context") &&
                ok(c, cuCtxSetCurrent(c->ctx), "cuCtxSetCurrent") && ok(c, cuModuleLoad(&c->mod, cubin), "cuModuleLoad");
    struct { CUfunction *f; const char *name; } fns[] = {
        {&c->k.identify, "_Z22cuda_identify_meetingsP9workbench"},
        {&c->k.init_o_boxs, "_Z16cuda_init_o_boxsP9workbench"},
        {&c->k.set_oid, "_Z7set_oidP9workbench"},
        {&c->k.get_o_limit, "_Z11get_o_limitP9workbenchj"},
        {&c->k.write_o_bitmap, "_Z19cuda_write_o_bitmapP9workbenchj"},
        {&c->k.narrow_xy_to_y, "_Z14narrow_xy_to_yP9workbench"},
        {&c->k.make_sid, "_Z8make_sidP9workbench"},
        {&c->k.write_sid_in_key, "_Z16write_sid_in_keyP9workbench"},
        {&c->k.get_ctf_capacity, "_Z16get_CTF_capacityP9workbench"},
        {&c->k.get_limit, "_Z14cuda_get_limitP9workbench"},
        {&c->k.write_bitmap, "_Z17cuda_write_bitmapP9workbench"},
        {&c->k.write_key_and_mbr, "_Z17write_key_and_mbrP9workbench"},
    };
    for (auto &f : fns)
        if (good) good = ok(c, cuModuleGetFunction(f.f, c->mod, f.name), f.name);
    const size_t N = c->N;
    if (good)
        good = alloc(c, &c->d_bench, RG_WB_SIZE) && alloc(c, &c->d_cfg, RG_CFG_SIZE) &&
               alloc(c, &c->d_keys, c->kv_capacity * 16) && alloc(c, &c->d_ctf_keys, c->kv_capacity * 16) &&
               alloc(c, &c->d_kv_boxs, c->kv_capacity * RG_F_BOX_SIZE) && alloc(c, &c->d_mid_xys, N * 8) &&
               alloc(c, &c->d_same, N * 4) && alloc(c, &c->d_sids, N * 2) && alloc(c, &c->d_o_boxs, N * RG_UINT_BOX_SIZE) &&
               alloc(c, &c->d_oids, N * 4) && alloc(c, &c->d_bitmaps, c->bitmaps_size + kBitmapSlack) &&
               alloc(c, &c->d_capacity, (size_t)c->CTF_count * 4) && alloc(c, &c->d_ctfs, (size_t)c->CTF_count * RG_CTF_SIZE);
    if (good) {
        put<uint32_t>(c->cfg, RG_CFG_num_objects, c->N);
        put<uint32_t>(c->cfg, RG_CFG_min_meet_time, c->min_meet_time);
        put<uint32_t>(c->cfg, RG_CFG_max_meet_time, c->max_meet_time);
        put<uint32_t>(c->cfg, RG_CFG_kv_capacity, (uint32_t)c->kv_capacity);
        put<uint32_t>(c->cfg, RG_CFG_CTF_count, c->CTF_count);
        put<uint32_t>(c->cfg, RG_CFG_split_num, c->split_num);
        put<uint32_t>(c->cfg, RG_CFG_search_multi_capacity, 0xffffffffu);
        put<uint32_t>(c->cfg, RG_CFG_search_single_capacity, 0xffffffffu);
        put<uint64_t>(c->wb, RG_WB_config, c->d_cfg);
        std::memcpy(c->wb.data() + RG_WB_mbr, c->mbr, RG_BOX_SIZE);  /* box: low[2], high[2] doubles */
        put<uint64_t>(c->wb, RG_WB_d_keys, c->d_keys);
        put<uint64_t>(c->wb, RG_WB_d_ctf_keys, c->d_ctf_keys);
        put<double>(c->wb, RG_WB_dProbFalse, cfg->dProbFalse);
        put<uint64_t>(c->wb, RG_WB_mid_xys, c->d_mid_xys);
        put<uint64_t>(c->wb, RG_WB_same_pid_count, c->d_same);
        put<uint64_t>(c->wb, RG_WB_d_sids, c->d_sids);
        put<uint64_t>(c->wb, RG_WB_kv_boxs, c->d_kv_boxs);
        put<uint64_t>(c->wb, RG_WB_o_boxs, c->d_o_boxs);
        put<uint64_t>(c->wb, RG_WB_d_bitmaps, c->d_bitmaps);
        put<uint32_t>(c->wb, RG_WB_bit_count, c->bit_count);
        put<uint32_t>(c->wb, RG_WB_bitmaps_size, c->bitmaps_size);
        put<uint64_t>(c->wb, RG_WB_d_oids, c->d_oids);
        put<uint64_t>(c->wb, RG_WB_d_CTF_capacity, c->d_capacity);
        put<uint64_t>(c->wb, RG_WB_d_ctfs, c->d_ctfs);
        good = bench_up(c) && reset_store(c);
    }
    *out = c;  /* also on failure, for rg_error; the caller closes it */
    return good ? 0 : -1;
}

const char *rg_error(const rg_ctx *c) { return c ? c->err.c_str() : "no context"; }

/* n meeting_unit records (the bucket layout: Cantor key, start, end, f32
 * box) through the reference's cuda_identify_meetings at cur_time, with the
 * active multi-search over pids when npids > 0; *found receives the
 * multi-search's record count and the first cap records go to out */
int rg_identify(rg_ctx *c, const void *units, uint64_t n, uint32_t cur_time, uint32_t end_time_min,
                const uint32_t *pids, uint32_t npids, go_search_info *out, uint64_t cap, uint64_t *found) {
    CUdeviceptr d_units = 0, d_list = 0, d_pids = 0;
    /* a bucket yields one record per listed occurrence of either id */
    uint64_t mult = 0;
    if (npids) {
        std::vector<uint32_t> p(pids, pids + npids);
        std::sort(p.begin(), p.end());
        for (size_t i = 0, j; i < p.size(); i = j) {
            for (j = i; j < p.size() && p[j] == p[i]; ++j) {}
            mult = std::max<uint64_t>(mult, j - i);
        }
    }
    const uint64_t list_cap = 2ull * n * mult + 1;
    if (!bench_down(c)) return -1;
    if ((uint64_t)get<uint32_t>(c->wb, RG_WB_kv_count) + 2 * n > c->kv_capacity) {
        c->err = "key buffer too small for these meetings (the reference asserts)";
        return -2;
    }
    bool good = alloc(c, &d_units, n * RG_MU_SIZE) && ok(c, cuMemcpyHtoD(d_units, units, n * RG_MU_SIZE), "units") &&
                alloc(c, &d_list, list_cap * RG_SIU_SIZE) && alloc(c, &d_pids, (size_t)npids * 4 + 4);
    if (good && npids) good = ok(c, cuMemcpyHtoD(d_pids, pids, (size_t)npids * 4), "pids");
    if (good) good = bench_down(c);
    if (good) {
        put<uint64_t>(c->cfg, RG_CFG_num_meeting_buckets, n);
        put<uint64_t>(c->wb, RG_WB_meeting_buckets, d_units);
        put<uint32_t>(c->wb, RG_WB_cur_time, cur_time);
        put<uint32_t>(c->wb, RG_WB_end_time_min, end_time_min);
        put<uint8_t>(c->wb, RG_WB_search_single, 0);
        put<uint8_t>(c->wb, RG_WB_search_multi, npids ? 1 : 0);
        put<uint64_t>(c->wb, RG_WB_search_multi_list, d_list);
        put<uint32_t>(c->wb, RG_WB_search_multi_length, npids);
        put<uint64_t>(c->wb, RG_WB_search_multi_pid, d_pids);
        put<uint32_t>(c->wb, RG_WB_multi_find_count, 0);
        good = bench_up(c) && launch(c, c->k.identify, n / 1024 + 1, 1024, "cuda_identify_meetings") && bench_down(c);
    }
    if (good) {
        const uint32_t nf = get<uint32_t>(c->wb, RG_WB_multi_find_count);
        if (found) *found = nf;
        const uint64_t take = std::min<uint64_t>(std::min<uint64_t>(nf, cap), list_cap);
        if (take && out) good = ok(c, cuMemcpyDtoH(out, d_list, take * RG_SIU_SIZE), "search list");
        put<uint64_t>(c->wb, RG_WB_meeting_buckets, 0);
        put<uint8_t>(c->wb, RG_WB_search_multi, 0);
        if (good) good = bench_up(c);
    }
    if (d_units) cuMemFree(d_units);
    if (d_list) cuMemFree(d_list);
    if (d_pids) cuMemFree(d_pids);
    return good ? 0 : -1;
}

/* the pending keys' count, objects with keys and oversize objects */
int rg_pending(rg_ctx *c, uint64_t *kv_count, uint32_t *sid_count, uint32_t *oversize_oid_count) {
    if (!bench_down(c)) return -1;
    *kv_count = get<uint32_t>(c->wb, RG_WB_kv_count);
    *sid_count = get<uint32_t>(c->wb, RG_WB_sid_count);
    *oversize_oid_count = get<uint32_t>(c->wb, RG_WB_oversize_oid_count);
    return 0;
}

/* process_with_gpu's "4.5 cuda sort" block (cuda/geometry.cu:1752-2135) at
 * cur_time, then the reset that follows it */
int rg_flush(rg_ctx *c, uint32_t cur_time, rg_flush_info *info) {
    const size_t N = c->N;
    const uint32_t C = c->CTF_count;
    if (!bench_down(c)) return -1;
    put<uint32_t>(c->wb, RG_WB_cur_time, cur_time);
    if (!bench_up(c)) return -1;
    if (!launch(c, c->k.set_oid, N / 1024 + 1, 1024, "set_oid") || !bench_down(c)) return -1;
    /* thrust::partition of (key, box) by sid != 1: a stable partition here */
    const uint32_t old_kv = get<uint32_t>(c->wb, RG_WB_kv_count);
    std::vector<u128> keys(old_kv);
    std::vector<uint8_t> boxes((size_t)old_kv * 16);
    std::vector<uint16_t> sids(N);
    if (old_kv && (!ok(c, cuMemcpyDtoH(keys.data(), c->d_keys, (size_t)old_kv * 16), "keys") ||
                   !ok(c, cuMemcpyDtoH(boxes.data(), c->d_kv_boxs, (size_t)old_kv * 16), "boxes")))
        return -1;
    if (!ok(c, cuMemcpyDtoH(sids.data(), c->d_sids, N * 2), "sids")) return -1;
    std::vector<u128> k2;
    std::vector<uint8_t> b2;
    k2.reserve(old_kv);
    b2.reserve((size_t)old_kv * 16);
    /* cuda_get_key_oid: the 26 bits above target, duration and end */
    auto key_oid = [](u128 k) { return (uint32_t)(k >> (26 + 32 + 32)) & ((1u << 26) - 1); };
    for (int pass = 0; pass < 2; ++pass)
        for (uint32_t i = 0; i < old_kv; ++i) {
            const bool keep = sids[key_oid(keys[i])] != 1;
            if (keep == (pass == 0)) {
                k2.push_back(keys[i]);
                b2.insert(b2.end(), &boxes[(size_t)i * 16], &boxes[(size_t)i * 16] + 16);
            }
        }
    uint32_t kv = 0;
    for (uint32_t i = 0; i < old_kv; ++i)
        if (sids[key_oid(keys[i])] != 1) ++kv;
    const uint32_t ov = old_kv - kv;
    if (old_kv && (!ok(c, cuMemcpyHtoD(c->d_keys, k2.data(), (size_t)old_kv * 16), "keys") ||
                   !ok(c, cuMemcpyHtoD(c->d_kv_boxs, b2.data(), (size_t)old_kv * 16), "boxes")))
        return -1;
    put<uint32_t>(c->wb, RG_WB_kv_count, kv);
    if (!bench_up(c)) return -1;
    if (!sort_by_key<u128>(c, c->d_keys + (size_t)kv * 16, c->d_kv_boxs + (size_t)kv * 16, ov, 16)) return -1;
    uint32_t ovc = ov;
    if (!launch(c, c->k.get_o_limit, 1, 1024, "get_o_limit", &ovc)) return -1;
    std::vector<uint8_t> ctf0(RG_CTF_SIZE);
    if (!ok(c, cuMemcpyDtoH(ctf0.data(), c->d_ctfs, RG_CTF_SIZE), "ctf 0")) return -1;
    const go_ctf_meta om = meta_of(ctf0.data());
    if (!launch(c, c->k.write_o_bitmap, ov / 1024 + 1, 1024, "cuda_write_o_bitmap", &ovc)) return -1;
    c->o_bitmap.assign(c->bit_count / 8, 0);
    if (!ok(c, cuMemcpyDtoH(c->o_bitmap.data(), c->d_bitmaps, c->bit_count / 8), "o bitmap") ||
        !ok(c, cuMemsetD8(c->d_bitmaps, 0, c->bit_count / 8), "o bitmap clear"))
        return -1;
    /* STR: mid_xys -> oids by x, then by y within each x slab (stable) */
    if (!sort_by_key<uint64_t>(c, c->d_mid_xys, c->d_oids, N, 4)) return -1;
    if (!launch(c, c->k.narrow_xy_to_y, N / 1024 + 1, 1024, "narrow_xy_to_y") || !bench_down(c)) return -1;
    const uint32_t sid_count = get<uint32_t>(c->wb, RG_WB_sid_count);
    const uint32_t ovo = get<uint32_t>(c->wb, RG_WB_oversize_oid_count);
    const uint64_t zero_one = (uint64_t)(N - sid_count) + ovo;
    const uint64_t xpc = (uint64_t)(sid_count - ovo) / c->split_num + 1;
    for (uint32_t i = 0; i < c->split_num; ++i) {
        const uint64_t b = std::min<uint64_t>(zero_one + xpc * i, N);
        const uint64_t e = i + 1 < c->split_num ? std::min<uint64_t>(zero_one + xpc * (i + 1), N) : N;
        if (e > b && !sort_by_key<uint64_t>(c, c->d_mid_xys + b * 8, c->d_oids + b * 4, e - b, 4)) return -1;
    }
    if (!launch(c, c->k.make_sid, N / 1024 + 1, 1024, "make_sid") ||
        !launch(c, c->k.write_sid_in_key, kv / 1024 + 1, 1024, "write_sid_in_key"))
        return -1;
    if (!sort_by_key<u128>(c, c->d_keys, c->d_kv_boxs, kv, 16)) return -1;
    if (!launch(c, c->k.get_ctf_capacity, N / 1024 + 1, 1024, "get_CTF_capacity") ||
        !launch(c, c->k.get_limit, C, 1024, "cuda_get_limit"))
        return -1;
    std::vector<uint8_t> img((size_t)C * RG_CTF_SIZE);
    if (!ok(c, cuMemcpyDtoH(img.data(), c->d_ctfs, img.size()), "ctfs")) return -1;
    c->ctfs.resize(C);
    for (uint32_t i = 0; i < C; ++i) {
        go_ctf_meta m = meta_of(&img[(size_t)i * RG_CTF_SIZE]);
        if (!go_ctf_bits(&m, c->mbr, c->N, c->max_meet_time)) {
            c->err = "get_ctf_bits would assert (a CTF outside the reference's domain)";
            return -2;
        }
        meta_into(&img[(size_t)i * RG_CTF_SIZE], m);
        c->ctfs[i] = m;
    }
    if (!ok(c, cuMemcpyHtoD(c->d_ctfs, img.data(), img.size()), "ctfs")) return -1;
    /* cuda_write_bitmap sets the cells a box covers relative to its CTF's box
     * with no bounds check; a box outside that box (the CTF box is a partial
     * reduction) reaches past the CTF's bitmap.  Bound every loop and bit
     * position, in double with a margin, before launching it. */
    {
        std::vector<uint32_t> cap(C);
        std::vector<float> bx((size_t)kv * 4);
        if (!ok(c, cuMemcpyDtoH(cap.data(), c->d_capacity, (size_t)C * 4), "capacity") ||
            (kv && !ok(c, cuMemcpyDtoH(bx.data(), c->d_kv_boxs, (size_t)kv * 16), "boxes")))
            return -1;
        const double limit_bits = 8.0 * ((double)c->bitmaps_size + kBitmapSlack);
        uint64_t kid = 0;
        for (uint32_t i = 0; i < C; ++i) {
            const go_ctf_meta &m = c->ctfs[i];
            const double w = (double)m.ctf_mbr[2] - m.ctf_mbr[0], h = (double)m.ctf_mbr[3] - m.ctf_mbr[1];
            for (uint32_t q = 0; q < cap[i]; ++q, ++kid) {
                if (kid >= kv) {
                    c->err = "CTF capacities exceed the key count";
                    return -3;
                }
                const float *b = &bx[kid * 4];  /* f_box: low[0], low[1], high[0], high[1] */
                const double lx = std::max(0.0, ((double)b[0] - m.ctf_mbr[0]) / w * m.x_grid);
                const double ly = std::max(0.0, ((double)b[1] - m.ctf_mbr[1]) / h * m.y_grid);
                const double hx = ((double)b[2] - m.ctf_mbr[0]) / w * m.x_grid;
                const double hy = ((double)b[3] - m.ctf_mbr[1]) / h * m.y_grid;
                const bool finite = w > 0 && h > 0 && hx < 1e5 && hy < 1e5;
                if (!finite || (hx - lx + 2) * (hy - ly + 2) > 1e7 ||
                    (double)i * c->bit_count + hx + 1 + (hy + 1) * m.x_grid >= limit_bits) {
                    c->err = "a key's box reaches too far from its CTF's box for the unchecked bitmap loop";
                    return -3;
                }
            }
        }
    }
    if (!launch(c, c->k.write_bitmap, C, 1024, "cuda_write_bitmap") ||
        !launch(c, c->k.write_key_and_mbr, C, 1024, "write_key_and_mbr"))
        return -1;
    /* outputs (cuda/geometry.cu:2020-2035) */
    c->capacity.assign(C, 0);
    if (!ok(c, cuMemcpyDtoH(c->capacity.data(), c->d_capacity, (size_t)C * 4), "capacity")) return -1;
    uint64_t key_bytes = 0;
    for (uint32_t i = 0; i < C; ++i) key_bytes += (uint64_t)c->capacity[i] * (c->ctfs[i].key_bit / 8);
    c->packed.assign(key_bytes, 0);
    c->sids.assign(N, 0);
    c->bitmaps.assign(c->bitmaps_size, 0);
    c->o_keys.assign(ov, 0);
    c->o_boxes.assign((size_t)ov * 4, 0);
    if ((key_bytes && !ok(c, cuMemcpyDtoH(c->packed.data(), c->d_ctf_keys, key_bytes), "packed")) ||
        !ok(c, cuMemcpyDtoH(c->sids.data(), c->d_sids, N * 2), "sids") ||
        !ok(c, cuMemcpyDtoH(c->bitmaps.data(), c->d_bitmaps, c->bitmaps_size), "bitmaps") ||
        (ov && !ok(c, cuMemcpyDtoH(c->o_keys.data(), c->d_keys + (size_t)kv * 16, (size_t)ov * 16), "o keys")) ||
        (ov && !ok(c, cuMemcpyDtoH(c->o_boxes.data(), c->d_kv_boxs + (size_t)kv * 16, (size_t)ov * 16), "o boxes")))
        return -1;
    /* bits that landed past the bitmap array, in the slack */
    std::vector<uint8_t> slack(kBitmapSlack);
    if (!ok(c, cuMemcpyDtoH(slack.data(), c->d_bitmaps + c->bitmaps_size, kBitmapSlack), "slack")) return -1;
    uint64_t outside = 0;
    for (uint8_t b : slack) outside += __builtin_popcount(b);
    std::memset(&c->info, 0, sizeof(c->info));
    c->info.kv_count = kv;
    c->info.key_bytes = key_bytes;
    c->info.oversize_kv_count = ov;
    c->info.oversize_start_time_min = om.start_time_min;
    c->info.oversize_start_time_max = om.start_time_max;
    c->info.oversize_end_time_min = om.end_time_min;
    c->info.oversize_end_time_max = om.end_time_max;
    c->info.sid_count = sid_count;
    c->info.oversize_oid_count = ovo;
    c->info.bits_in_slack = outside;
    if (info) *info = c->info;
    return reset_store(c) ? 0 : -1;
}

void rg_result(const rg_ctx *c, uint8_t *keys, uint16_t *sids, uint32_t *ctf_capacity, go_ctf_meta *ctfs,
               uint8_t *bitmaps, void *o_keys, float *o_boxes, uint8_t *o_bitmap) {
    if (keys) std::memcpy(keys, c->packed.data(), c->packed.size());
    if (sids) std::memcpy(sids, c->sids.data(), c->sids.size() * 2);
    if (ctf_capacity) std::memcpy(ctf_capacity, c->capacity.data(), c->capacity.size() * 4);
    if (ctfs) std::memcpy(ctfs, c->ctfs.data(), c->ctfs.size() * sizeof(go_ctf_meta));
    if (bitmaps) std::memcpy(bitmaps, c->bitmaps.data(), c->bitmaps.size());
    if (o_keys) std::memcpy(o_keys, c->o_keys.data(), c->o_keys.size() * 16);
    if (o_boxes) std::memcpy(o_boxes, c->o_boxes.data(), c->o_boxes.size() * 4);
    if (o_bitmap) std::memcpy(o_bitmap, c->o_bitmap.data(), c->o_bitmap.size());
}

void rg_close(rg_ctx *c) {
    if (!c) return;
    CUdeviceptr ps[] = {c->d_bench, c->d_cfg, c->d_keys, c->d_ctf_keys, c->d_kv_boxs, c->d_mid_xys, c->d_same,
                        c->d_sids, c->d_o_boxs, c->d_oids, c->d_bitmaps, c->d_capacity, c->d_ctfs};
    for (CUdeviceptr p : ps)
        if (p) cuMemFree(p);
    if (c->mod) cuModuleUnload(c->mod);
    if (c->ctx) cuDevicePrimaryCtxRelease(c->dev);
    delete c;
}

}  // extern "C"
