/*
 * store_files.cu -- a flushed block on disk in the reference's file layout,
 * and back onto the device for queries.
 *
 * Writing follows straight_dump (tracing/process.cpp:254-348), which for
 * block `ctb` writes
 *   <raid_path><i % 2>/<prefix>_SSTable_<ctb>-<i>   CTF i's packed keys
 *   <meta_path>/<prefix>_CTB<ctb>                   the CTB record, sids,
 *       oversize keys, boxes and bitmap (workbench::dump_CTB_meta,
 *       tracing/workbench.cpp:597-614)
 *   <meta_path>/<prefix>_STcL<ctb>-<i>              the CTF record and the
 *       first ctf_bitmap_size bytes of its bitmap (CTF::dump_meta,
 *       tracing/step_merge.cpp:644-650)
 * and reading follows workbench::load_CTB_meta / load_CTF_meta /
 * load_CTF_keys (tracing/workbench.cpp:302-325, 639-695).  The records are
 * the reference's classes written whole with ofstream::write, so their LP64
 * layouts (CTF 80 bytes, oversize_buffer 48, CTB 128) are restated here.  The
 * reference writes its heap addresses into the pointer fields and its loader
 * overwrites them; here they are written as zero.  straight_dump leaves the
 * CTB's own count and time fields zero, and so does this writer for a
 * flushed block; a compacted block carries the time fields merge_dump
 * folds (tools/compaction.cpp:966-976) and a CTF count of zero, as
 * merge_dump leaves it.
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "glint_internal.cuh"

namespace {

constexpr uint32_t kBitmapBytes = 256 * 256 / 8; /* DEFAULT_bitmap_edge^2 bits, util/util.h:47 */
constexpr int kOidBits = 26;                     /* OID_BIT, util/util.h:49 */

/* class CTF (tracing/step_merge.h:67-110) as written by CTF::dump_meta */
struct FileCTF {
    float ctf_mbr[4];
    uint64_t keys_ptr;
    uint64_t bitmap_ptr;
    uint32_t CTF_kv_capacity, start_time_min, start_time_max, end_time_min, end_time_max, ctf_bitmap_size;
    uint16_t key_bit, id_bit, duration_bit, end_bit, low_x_bit, low_y_bit, edge_bit, mbr_bit, x_grid, y_grid;
    uint32_t pad;
};
static_assert(sizeof(FileCTF) == 80, "CTF record");
static_assert(offsetof(FileCTF, CTF_kv_capacity) == 32 && offsetof(FileCTF, key_bit) == 56, "CTF fields");

/* class oversize_buffer (tracing/step_merge.h:45-61) */
struct FileOBuffer {
    uint32_t oversize_kv_count, pad;
    uint64_t keys_ptr, boxes_ptr, o_bitmaps_ptr;
    uint32_t start_time_min, start_time_max, end_time_min, end_time_max;
};
static_assert(sizeof(FileOBuffer) == 48, "oversize_buffer record");

/* class CTB (tracing/step_merge.h:111-131) as written by dump_CTB_meta */
struct FileCTB {
    uint64_t ctfs_ptr;
    uint32_t CTF_count, start_time_min, start_time_max, end_time_min, end_time_max, pad;
    uint64_t first_widpid_ptr, sids_ptr, bitmaps_ptr, bitmap_mbrs_ptr, CTF_capacity_ptr;
    FileOBuffer o_buffer;
    uint64_t box_rtree_ptr;
};
static_assert(sizeof(FileCTB) == 128 && offsetof(FileCTB, o_buffer) == 72, "CTB record");

struct Paths {
    std::string raid, meta, prefix;
    uint32_t ctb;
    std::string sstable(uint32_t i) const {
        return raid + std::to_string(i % 2) + "/" + prefix + "_SSTable_" + std::to_string(ctb) + "-" + std::to_string(i);
    }
    std::string ctb_meta() const { return meta + "/" + prefix + "_CTB" + std::to_string(ctb); }
    std::string ctf_meta(uint32_t i) const {
        return meta + "/" + prefix + "_STcL" + std::to_string(ctb) + "-" + std::to_string(i);
    }
};

/* the last failure of a call that has no context */
thread_local std::string g_file_error;

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

bool write_file(const std::string &path, const std::vector<std::pair<const void *, size_t>> &parts, std::string &err) {
    File out;
    out.f = fopen(path.c_str(), "wb");
    if (!out.f) {
        err = "cannot create " + path;
        return false;
    }
    for (const auto &p : parts)
        if (p.second && fwrite(p.first, 1, p.second, out.f) != p.second) {
            err = "short write to " + path;
            return false;
        }
    if (fclose(out.f) != 0) {
        out.f = nullptr;
        err = "cannot close " + path;
        return false;
    }
    out.f = nullptr;
    return true;
}

bool read_exact(FILE *f, void *dst, size_t n) { return n == 0 || fread(dst, 1, n, f) == n; }

glint_status write_store(const glint_store_view &v, const Paths &p, std::string &err,
                         const uint32_t *rec_times = nullptr) {
    const uint32_t C = v.CTF_count, N = v.num_objects;
    /* SSTables: CTF after CTF in the packed key buffer */
    uint64_t at = 0;
    for (uint32_t i = 0; i < C; ++i) {
        const uint64_t n = (uint64_t)v.ctfs[i].CTF_kv_capacity * (v.ctfs[i].key_bit / 8);
        if (at + n > v.info.key_bytes) {
            err = "CTF capacities exceed the packed key bytes";
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        if (!write_file(p.sstable(i), {{v.keys + at, n}}, err)) return GLINT_ERR_INVALID_ARGUMENT;
        at += n;
    }
    /* CTB record, sids, oversize keys, boxes, bitmap */
    FileCTB ctb;
    std::memset(&ctb, 0, sizeof(ctb));
    if (rec_times) {
        ctb.start_time_min = rec_times[0];
        ctb.start_time_max = rec_times[1];
        ctb.end_time_min = rec_times[2];
        ctb.end_time_max = rec_times[3];
    }
    const uint32_t on = v.info.oversize_kv_count;
    ctb.o_buffer.oversize_kv_count = on;
    ctb.o_buffer.start_time_min = v.info.oversize_start_time_min;
    ctb.o_buffer.start_time_max = v.info.oversize_start_time_max;
    ctb.o_buffer.end_time_min = v.info.oversize_end_time_min;
    ctb.o_buffer.end_time_max = v.info.oversize_end_time_max;
    if (!write_file(p.ctb_meta(),
                    {{&ctb, sizeof(ctb)},
                     {v.sids, sizeof(uint16_t) * (size_t)N},
                     {v.oversize_keys, (size_t)16 * on},
                     {v.oversize_boxes, sizeof(float) * 4 * (size_t)on},
                     {v.oversize_bitmap, kBitmapBytes}},
                    err))
        return GLINT_ERR_INVALID_ARGUMENT;
    /* CTF records and their bitmaps */
    for (uint32_t i = 0; i < C; ++i) {
        const glint_ctf_meta &m = v.ctfs[i];
        if (m.ctf_bitmap_size > kBitmapBytes) {
            err = "CTF bitmap larger than its slot";
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        FileCTF r;
        std::memset(&r, 0, sizeof(r));
        std::memcpy(r.ctf_mbr, m.ctf_mbr, sizeof(r.ctf_mbr));
        r.CTF_kv_capacity = m.CTF_kv_capacity;
        r.start_time_min = m.start_time_min;
        r.start_time_max = m.start_time_max;
        r.end_time_min = m.end_time_min;
        r.end_time_max = m.end_time_max;
        r.ctf_bitmap_size = m.ctf_bitmap_size;
        r.key_bit = m.key_bit;
        r.id_bit = m.id_bit;
        r.duration_bit = m.duration_bit;
        r.end_bit = m.end_bit;
        r.low_x_bit = m.low_x_bit;
        r.low_y_bit = m.low_y_bit;
        r.edge_bit = m.edge_bit;
        r.mbr_bit = m.mbr_bit;
        r.x_grid = m.x_grid;
        r.y_grid = m.y_grid;
        if (!write_file(p.ctf_meta(i), {{&r, sizeof(r)}, {v.bitmaps + (size_t)i * kBitmapBytes, m.ctf_bitmap_size}},
                        err))
            return GLINT_ERR_INVALID_ARGUMENT;
    }
    return GLINT_OK;
}

/* a block read back from files, on the host */
struct HostBlock {
    std::vector<uint8_t> keys;
    std::vector<glint_ctf_meta> ctfs;
    std::vector<unsigned long long> key_index, byte_index;
    std::vector<uint16_t> sids;
    std::vector<uint32_t> first, count;
    std::vector<ulonglong2> okeys;
    std::vector<float4> oboxes;
    std::vector<uint8_t> bitmaps, obitmap;
    uint64_t kv = 0;
    uint32_t end_time_min = 0, end_time_max = 0;
    uint32_t o_times[4] = {0, 0, 0, 0}, rec_times[4] = {0, 0, 0, 0};
};

glint_status read_store(const Paths &p, uint32_t N, uint32_t C, HostBlock &h, std::string &err) {
    /* CTB record, sids, oversize keys, boxes and bitmap */
    {
        File in;
        in.f = fopen(p.ctb_meta().c_str(), "rb");
        if (!in.f) {
            err = "cannot open " + p.ctb_meta();
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        FileCTB ctb;
        h.sids.resize(N);
        if (!read_exact(in.f, &ctb, sizeof(ctb)) || !read_exact(in.f, h.sids.data(), sizeof(uint16_t) * (size_t)N)) {
            err = "short CTB file " + p.ctb_meta();
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        h.okeys.resize(ctb.o_buffer.oversize_kv_count);
        h.oboxes.resize(ctb.o_buffer.oversize_kv_count);
        h.obitmap.resize(kBitmapBytes);
        if (!read_exact(in.f, h.okeys.data(), 16 * h.okeys.size()) ||
            !read_exact(in.f, h.oboxes.data(), sizeof(float4) * h.oboxes.size()) ||
            !read_exact(in.f, h.obitmap.data(), kBitmapBytes)) {
            err = "short CTB file " + p.ctb_meta();
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        h.end_time_min = ctb.o_buffer.end_time_min;
        h.end_time_max = ctb.o_buffer.end_time_max;
        h.o_times[0] = ctb.o_buffer.start_time_min;
        h.o_times[1] = ctb.o_buffer.start_time_max;
        h.o_times[2] = ctb.o_buffer.end_time_min;
        h.o_times[3] = ctb.o_buffer.end_time_max;
        h.rec_times[0] = ctb.start_time_min;
        h.rec_times[1] = ctb.start_time_max;
        h.rec_times[2] = ctb.end_time_min;
        h.rec_times[3] = ctb.end_time_max;
    }
    /* CTF records and their bitmaps */
    h.ctfs.resize(C);
    h.key_index.resize(C);
    h.byte_index.resize(C);
    h.bitmaps.assign((size_t)C * kBitmapBytes, 0);
    uint64_t kv = 0, bytes = 0;
    for (uint32_t i = 0; i < C; ++i) {
        File in;
        in.f = fopen(p.ctf_meta(i).c_str(), "rb");
        FileCTF r;
        if (!in.f || !read_exact(in.f, &r, sizeof(r))) {
            err = "cannot read " + p.ctf_meta(i);
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        glint_ctf_meta &m = h.ctfs[i];
        std::memset(&m, 0, sizeof(m));
        std::memcpy(m.ctf_mbr, r.ctf_mbr, sizeof(m.ctf_mbr));
        m.CTF_kv_capacity = r.CTF_kv_capacity;
        m.start_time_min = r.start_time_min;
        m.start_time_max = r.start_time_max;
        m.end_time_min = r.end_time_min;
        m.end_time_max = r.end_time_max;
        m.ctf_bitmap_size = r.ctf_bitmap_size;
        m.key_bit = r.key_bit;
        m.id_bit = r.id_bit;
        m.duration_bit = r.duration_bit;
        m.end_bit = r.end_bit;
        m.low_x_bit = r.low_x_bit;
        m.low_y_bit = r.low_y_bit;
        m.edge_bit = r.edge_bit;
        m.mbr_bit = r.mbr_bit;
        m.x_grid = r.x_grid;
        m.y_grid = r.y_grid;
        if (m.key_bit == 0 || m.key_bit % 8 || m.key_bit > 128 || m.id_bit == 0 || m.id_bit > 32 ||
            m.ctf_bitmap_size > kBitmapBytes) {
            err = "CTF record out of range in " + p.ctf_meta(i);
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        if (!read_exact(in.f, h.bitmaps.data() + (size_t)i * kBitmapBytes, m.ctf_bitmap_size)) {
            err = "short CTF file " + p.ctf_meta(i);
            return GLINT_ERR_INVALID_ARGUMENT;
        }
        h.key_index[i] = kv;
        h.byte_index[i] = bytes;
        kv += m.CTF_kv_capacity;
        bytes += (uint64_t)m.CTF_kv_capacity * (m.key_bit / 8);
    }
    h.kv = kv;
    /* SSTables */
    h.keys.resize(bytes);
    for (uint32_t i = 0; i < C; ++i) {
        const uint64_t n = (uint64_t)h.ctfs[i].CTF_kv_capacity * (h.ctfs[i].key_bit / 8);
        File in;
        in.f = fopen(p.sstable(i).c_str(), "rb");
        if (!in.f || !read_exact(in.f, h.keys.data() + h.byte_index[i], n)) {
            err = "cannot read " + p.sstable(i);
            return GLINT_ERR_INVALID_ARGUMENT;
        }
    }
    /* each object's keys: its sid picks its CTF (sid - 2) or the oversize
     * buffer (sid 1); CTF keys are sorted by oid (CTF::ctf_get_key_oid,
     * tracing/step_merge.cpp:331-333), oversize keys by the full key */
    h.first.assign(N, 0);
    h.count.assign(N, 0);
    for (uint32_t i = 0; i < C; ++i) {
        const glint_ctf_meta &m = h.ctfs[i];
        const uint32_t kb = m.key_bit / 8;
        const int shift = m.id_bit + m.duration_bit + m.end_bit + m.mbr_bit;
        const unsigned __int128 mask = ((unsigned __int128)1 << m.id_bit) - 1;
        const uint8_t *base = h.keys.data() + h.byte_index[i];
        for (uint32_t j = 0; j < m.CTF_kv_capacity; ++j) {
            unsigned __int128 v = 0;
            for (uint32_t t = 0; t < kb; ++t) v |= (unsigned __int128)base[(size_t)j * kb + t] << (8 * t);
            const uint32_t oid = shift < 128 ? (uint32_t)((v >> shift) & mask) : 0u;
            if (oid >= N || h.sids[oid] != i + 2) continue;
            if (h.count[oid] == 0) h.first[oid] = (uint32_t)(h.key_index[i] + j);
            ++h.count[oid];
        }
    }
    for (size_t j = 0; j < h.okeys.size(); ++j) {
        /* [sid:12][pid:26][target:26][duration:32][end:32]: pid sits above
         * the target in the high word */
        const uint32_t oid = (uint32_t)(h.okeys[j].y >> kOidBits) & ((1u << kOidBits) - 1);
        if (oid >= N || h.sids[oid] != 1) continue;
        if (h.count[oid] == 0) h.first[oid] = (uint32_t)j;
        ++h.count[oid];
    }
    return GLINT_OK;
}

} // namespace

using namespace glint;

extern "C" glint_status glint_store_write(const glint_store_view *v, const char *raid_path, const char *meta_path,
                                          const char *prefix, uint32_t ctb) {
    if (!v || !raid_path || !meta_path || !prefix || !v->ctfs || !v->sids || !v->bitmaps || !v->oversize_bitmap ||
        (v->info.key_bytes && !v->keys) ||
        (v->info.oversize_kv_count && (!v->oversize_keys || !v->oversize_boxes))) {
        g_file_error = "store write: missing argument";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    std::string err;
    const glint_status st = write_store(*v, Paths{raid_path, meta_path, prefix, ctb}, err);
    g_file_error = st == GLINT_OK ? std::string() : "store write: " + err;
    return st;
}

extern "C" const char *glint_store_file_error(void) { return g_file_error.c_str(); }

extern "C" glint_status glint_store_dump(glint_ctx *c, const char *raid_path, const char *meta_path,
                                         const char *prefix, uint32_t ctb) {
    if (!c || !raid_path || !meta_path || !prefix) return GLINT_ERR_INVALID_ARGUMENT;
    if (!c->store_valid) {
        c->last_error = "store dump: no flush yet";
        return GLINT_ERR_STATE;
    }
    const uint32_t C = c->cfg.CTF_count, N = c->N;
    glint_store_info info;
    glint_status st = glint_store_read(c, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &info);
    if (st != GLINT_OK) return st;
    std::vector<uint8_t> keys(info.key_bytes ? info.key_bytes : 1), bitmaps((size_t)C * kBitmapBytes),
        obitmap(kBitmapBytes), okeys((size_t)16 * info.oversize_kv_count + 16);
    std::vector<uint16_t> sids(N ? N : 1);
    std::vector<uint32_t> cap(C);
    std::vector<glint_ctf_meta> ctfs(C);
    std::vector<float> oboxes((size_t)4 * info.oversize_kv_count + 4);
    st = glint_store_read(c, keys.data(), sids.data(), cap.data(), ctfs.data(), bitmaps.data(), okeys.data(),
                          oboxes.data(), obitmap.data(), &info);
    if (st != GLINT_OK) return st;
    glint_store_view v;
    std::memset(&v, 0, sizeof(v));
    v.num_objects = N;
    v.CTF_count = C;
    v.keys = keys.data();
    v.sids = sids.data();
    v.ctfs = ctfs.data();
    v.bitmaps = bitmaps.data();
    v.oversize_keys = okeys.data();
    v.oversize_boxes = oboxes.data();
    v.oversize_bitmap = obitmap.data();
    v.info = info;
    std::string err;
    st = write_store(v, Paths{raid_path, meta_path, prefix, ctb}, err);
    if (st != GLINT_OK) c->last_error = "store dump: " + err;
    return st;
}

/* a block into the context's kept blocks (the oldest dropped beyond
 * store_keep) */
static glint_status keep_block(glint_ctx *c, StoreBlock &b) {
    c->ctbs.push_back(b);
    const cudaError_t e = store_blocks_trim(c);
    if (e != cudaSuccess) {
        c->last_error = std::string("store load: keeping the block: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    return GLINT_OK;
}

extern "C" glint_status glint_store_load_ctfs(glint_ctx *c, const char *raid_path, const char *meta_path,
                                              const char *prefix, uint32_t ctb, uint32_t ctf_count) {
    if (!c || !raid_path || !meta_path || !prefix || ctf_count == 0) return GLINT_ERR_INVALID_ARGUMENT;
    if (c->cfg.store_keep == 0) {
        c->last_error = "store load: the context keeps no blocks (store_keep = 0)";
        return GLINT_ERR_STATE;
    }
    const uint32_t C = ctf_count, N = c->N;
    HostBlock h;
    std::string err;
    glint_status st = read_store(Paths{raid_path, meta_path, prefix, ctb}, N, C, h, err);
    if (st != GLINT_OK) {
        c->last_error = "store load: " + err;
        return st;
    }
    /* the window base: every CTF record and the oversize buffer carry it */
    if (C) h.end_time_min = h.ctfs[0].end_time_min;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    cudaError_t e = cudaStreamSynchronize(s);
    StoreBlock b;
    auto A = [&](void **p, size_t n) {
        if (e == cudaSuccess) e = cudaMalloc(p, n ? n : 1);
    };
    A((void **)&b.keys, h.keys.size());
    A((void **)&b.ctfs, sizeof(glint_ctf_meta) * C);
    A((void **)&b.key_index, sizeof(unsigned long long) * C);
    A((void **)&b.byte_index, sizeof(unsigned long long) * C);
    A((void **)&b.sids, sizeof(uint16_t) * N);
    A((void **)&b.first, sizeof(uint32_t) * N);
    A((void **)&b.count, sizeof(uint32_t) * N);
    A((void **)&b.okeys, sizeof(ulonglong2) * h.okeys.size());
    A((void **)&b.oboxes, sizeof(float4) * h.oboxes.size());
    A((void **)&b.bitmaps, h.bitmaps.size());
    A((void **)&b.obitmap, h.obitmap.size());
    auto up = [&](void *dst, const void *src, size_t n) {
        if (e == cudaSuccess && n) e = cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice);
    };
    up(b.keys, h.keys.data(), h.keys.size());
    up(b.ctfs, h.ctfs.data(), sizeof(glint_ctf_meta) * C);
    up(b.key_index, h.key_index.data(), sizeof(unsigned long long) * C);
    up(b.byte_index, h.byte_index.data(), sizeof(unsigned long long) * C);
    up(b.sids, h.sids.data(), sizeof(uint16_t) * N);
    up(b.first, h.first.data(), sizeof(uint32_t) * N);
    up(b.count, h.count.data(), sizeof(uint32_t) * N);
    up(b.okeys, h.okeys.data(), sizeof(ulonglong2) * h.okeys.size());
    up(b.oboxes, h.oboxes.data(), sizeof(float4) * h.oboxes.size());
    up(b.bitmaps, h.bitmaps.data(), h.bitmaps.size());
    up(b.obitmap, h.obitmap.data(), h.obitmap.size());
    if (e != cudaSuccess) {
        store_block_release(b);
        c->last_error = std::string("store load: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
    }
    b.kv = h.kv;
    b.o_count = h.okeys.size();
    b.key_bytes = h.keys.size();
    b.end_time_min = h.end_time_min;
    b.end_time_max = h.end_time_max;
    b.C = C;
    std::memcpy(b.o_times, h.o_times, sizeof(b.o_times));
    std::memcpy(b.rec_times, h.rec_times, sizeof(b.rec_times));
    for (uint32_t o = 0; o < N; ++o) {
        b.sid_count += h.sids[o] >= 2;
        b.oversize_oid_count += h.sids[o] == 1;
    }
    return keep_block(c, b);
}

extern "C" glint_status glint_store_load(glint_ctx *c, const char *raid_path, const char *meta_path,
                                         const char *prefix, uint32_t ctb) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    return glint_store_load_ctfs(c, raid_path, meta_path, prefix, ctb, c->cfg.CTF_count);
}

extern "C" glint_status glint_store_block_info(glint_ctx *c, uint32_t block, glint_block_info *info) {
    if (!c || !info) return GLINT_ERR_INVALID_ARGUMENT;
    if (block >= c->ctbs.size()) {
        c->last_error = "block info: no such kept block";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    const StoreBlock &b = c->ctbs[block];
    std::memset(info, 0, sizeof(*info));
    info->CTF_count = b.C;
    std::memcpy(info->times, b.rec_times, sizeof(info->times));
    glint_store_info &st = info->store;
    st.kv_count = b.kv;
    st.key_bytes = b.key_bytes;
    st.oversize_kv_count = (uint32_t)b.o_count;
    st.oversize_start_time_min = b.o_times[0];
    st.oversize_start_time_max = b.o_times[1];
    st.oversize_end_time_min = b.o_times[2];
    st.oversize_end_time_max = b.o_times[3];
    st.sid_count = b.sid_count;
    st.oversize_oid_count = b.oversize_oid_count;
    st.end_time_min = b.end_time_min;
    st.cur_time = b.end_time_max;
    return GLINT_OK;
}

extern "C" glint_status glint_store_block_read(glint_ctx *c, uint32_t block, uint8_t *keys, uint16_t *sids,
                                               glint_ctf_meta *ctfs, uint8_t *bitmaps, void *oversize_keys,
                                               float *oversize_boxes, uint8_t *oversize_bitmap) {
    if (!c) return GLINT_ERR_INVALID_ARGUMENT;
    if (block >= c->ctbs.size()) {
        c->last_error = "block read: no such kept block";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    const StoreBlock &b = c->ctbs[block];
    auto down = [&](void *dst, const void *src, size_t n) {
        if (e == cudaSuccess && dst && n) e = cudaMemcpy(dst, src, n, cudaMemcpyDefault);
    };
    down(keys, b.keys, b.key_bytes);
    down(sids, b.sids, sizeof(uint16_t) * (size_t)c->N);
    down(ctfs, b.ctfs, sizeof(glint_ctf_meta) * b.C);
    down(bitmaps, b.bitmaps, (size_t)b.C * kBitmapBytes);
    down(oversize_keys, b.okeys, sizeof(ulonglong2) * b.o_count);
    down(oversize_boxes, b.oboxes, sizeof(float4) * b.o_count);
    down(oversize_bitmap, b.obitmap, kBitmapBytes);
    if (e != cudaSuccess) {
        c->last_error = std::string("block read: ") + cudaGetErrorString(e);
        return GLINT_ERR_CUDA;
    }
    return GLINT_OK;
}

extern "C" glint_status glint_store_block_dump(glint_ctx *c, uint32_t block, const char *raid_path,
                                               const char *meta_path, const char *prefix, uint32_t ctb) {
    if (!c || !raid_path || !meta_path || !prefix) return GLINT_ERR_INVALID_ARGUMENT;
    glint_block_info bi;
    glint_status st = glint_store_block_info(c, block, &bi);
    if (st != GLINT_OK) return st;
    const uint32_t C = bi.CTF_count, N = c->N;
    const glint_store_info &info = bi.store;
    std::vector<uint8_t> keys(info.key_bytes ? info.key_bytes : 1), bitmaps((size_t)C * kBitmapBytes),
        obitmap(kBitmapBytes), okeys((size_t)16 * info.oversize_kv_count + 16);
    std::vector<uint16_t> sids(N ? N : 1);
    std::vector<glint_ctf_meta> ctfs(C ? C : 1);
    std::vector<float> oboxes((size_t)4 * info.oversize_kv_count + 4);
    st = glint_store_block_read(c, block, keys.data(), sids.data(), ctfs.data(), bitmaps.data(), okeys.data(),
                                oboxes.data(), obitmap.data());
    if (st != GLINT_OK) return st;
    glint_store_view v;
    std::memset(&v, 0, sizeof(v));
    v.num_objects = N;
    v.CTF_count = C;
    v.keys = keys.data();
    v.sids = sids.data();
    v.ctfs = ctfs.data();
    v.bitmaps = bitmaps.data();
    v.oversize_keys = okeys.data();
    v.oversize_boxes = oboxes.data();
    v.oversize_bitmap = obitmap.data();
    v.info = info;
    std::string err;
    st = write_store(v, Paths{raid_path, meta_path, prefix, ctb}, err, bi.times);
    if (st != GLINT_OK) c->last_error = "block dump: " + err;
    return st;
}
