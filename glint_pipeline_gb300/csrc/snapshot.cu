/*
 * snapshot.cu -- saving a context between steps and resuming from the file.
 *
 * The reference dumps its workbench and CTB metadata (workbench::dump_meta,
 * tracing/workbench.cpp:574-596) and reloads them with load_meta
 * (tracing/process.cpp:213-236), but its meeting buckets, pending keys and
 * schema counters are not in that dump, so a resumed run loses the meetings
 * in progress.  A snapshot here holds everything the next steps read: the
 * schema (nodes, boxes, both free stacks, the last step's grid counts), the
 * meeting table (its occupied buckets), the pending keys of the current
 * window with their per-object counts, boxes and sids, the last step's
 * meetings, the last flushed store and the blocks kept for queries, and the
 * persistent counters.  A context resumed from it continues bit for bit as
 * the saved one would.
 *
 * File: a header record, then tagged sections (tag, byte count, bytes).
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "glint_internal.cuh"

using namespace glint;

namespace {

constexpr uint64_t kMagic = 0x31504E5354494C47ull; /* "GLITSNP1" */
constexpr uint64_t kTableChunk = 1ull << 22;        /* buckets per transfer */
constexpr uint32_t kVersion = 2;                    /* 2: kept blocks carry bitmaps, oversize boxes, times */
constexpr size_t kBitBytes = 65536 / 8;

/* a kept block's scalar fields */
struct SnapBlock {
    uint64_t kv, o_count, key_bytes;
    uint32_t end_time_min, end_time_max, C, sid_count;
    uint32_t o_times[4], rec_times[4];
    uint32_t oversize_oid_count, reserved;
};

struct SnapHeader {
    uint64_t magic;
    uint32_t version, header_bytes;
    glint_config cfg;
    glint_box mbr;
    uint64_t step_index;
    uint32_t last_time, end_time_min, flushes, store_valid;
    uint32_t num_blocks, reserved;
    uint64_t table_entries;
    DevCounters counters;
    glint_store_info store;
    glint_step_stats last_stats;
};

enum : uint32_t {
    kSecNodes = 1, kSecLow, kSecIbox, kSecSstack, kSecGstack, kSecGridCount, kSecOrder, kSecTable, kSecKeys,
    kSecKvBox, kSecSame, kSecObox, kSecSids, kSecMeetings, kSecStoreKeys, kSecStoreBoxes, kSecCtfKeys,
    kSecSidsOut, kSecCtfs, kSecBitmaps, kSecObitmap, kSecCtfCap, kSecBlock
};

struct Writer {
    FILE *f = nullptr;
    bool ok = true;
    void raw(const void *p, size_t n) {
        if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
    }
    void section(uint32_t tag, uint64_t bytes) {
        raw(&tag, sizeof(tag));
        raw(&bytes, sizeof(bytes));
    }
    /* a device array as one section */
    cudaError_t dev(uint32_t tag, const void *d, size_t bytes) {
        section(tag, bytes);
        std::vector<uint8_t> h(bytes);
        cudaError_t e = bytes ? cudaMemcpy(h.data(), d, bytes, cudaMemcpyDefault) : cudaSuccess;
        raw(h.data(), bytes);
        return e;
    }
};

struct Reader {
    FILE *f = nullptr;
    bool ok = true;
    void raw(void *p, size_t n) {
        if (ok && n && fread(p, 1, n, f) != n) ok = false;
    }
    bool section(uint32_t want, uint64_t &bytes) {
        uint32_t tag = 0;
        raw(&tag, sizeof(tag));
        raw(&bytes, sizeof(bytes));
        if (!ok || tag != want) ok = false;
        return ok;
    }
    cudaError_t dev(uint32_t tag, void *d, size_t expect) {
        uint64_t bytes = 0;
        if (!section(tag, bytes) || bytes != expect) {
            ok = false;
            return cudaSuccess;
        }
        std::vector<uint8_t> h(bytes);
        raw(h.data(), bytes);
        return (ok && bytes) ? cudaMemcpy(d, h.data(), bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    }
    /* a section into a fresh device allocation */
    cudaError_t dev_alloc(uint32_t tag, void **d, size_t expect) {
        cudaError_t e = cudaMalloc(d, expect ? expect : 1);
        if (e != cudaSuccess) return e;
        return dev(tag, *d, expect);
    }
};

__global__ void k_table_scatter(TRec *tab, uint8_t *stamp, const unsigned long long *slots, const TRec *recs,
                                uint64_t n, uint64_t B) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long s = slots[i];
        if (s >= B) continue;
        tab[s] = recs[i];
        stamp[s] = kStampOld;
    }
}

glint_status snap_fail(glint_ctx *c, cudaError_t e) {
    c->last_error = std::string("snapshot: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA;
}

} // namespace

extern "C" glint_status glint_snapshot_save(glint_ctx *c, const char *path) {
    if (!c || !path) return GLINT_ERR_INVALID_ARGUMENT;
    if (serve_only_refused(c, "snapshot")) return GLINT_ERR_STATE;
    if (c->step_index == 0) {
        c->last_error = "snapshot: before the first step";
        return GLINT_ERR_STATE;
    }
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return snap_fail(c, e);
    Writer w;
    w.f = fopen(path, "wb");
    if (!w.f) {
        c->last_error = std::string("snapshot: cannot create ") + path;
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    const uint32_t N = c->N, C = c->cfg.CTF_count;
    SnapHeader h;
    std::memset(&h, 0, sizeof(h));
    h.magic = kMagic;
    h.version = kVersion;
    h.header_bytes = sizeof(SnapHeader);
    h.cfg = c->cfg;
    h.mbr = c->mbr;
    h.step_index = c->step_index;
    h.last_time = c->last_time;
    h.end_time_min = c->end_time_min;
    h.flushes = c->flushes;
    h.store_valid = c->store_valid ? 1u : 0u;
    h.num_blocks = (uint32_t)c->ctbs.size();
    if (e == cudaSuccess) e = cudaMemcpy(&h.counters, c->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost);
    h.store = c->store;
    h.last_stats = c->last_stats;
    /* occupied buckets, counted first */
    std::vector<TRec> tb;
    std::vector<unsigned long long> slots;
    std::vector<TRec> recs;
    for (uint64_t b = 0; b < c->B && e == cudaSuccess; b += kTableChunk) {
        const uint64_t n = std::min<uint64_t>(kTableChunk, c->B - b);
        tb.resize(n);
        e = cudaMemcpy(tb.data(), c->d_tab + b, sizeof(TRec) * n, cudaMemcpyDeviceToHost);
        for (uint64_t i = 0; i < n; ++i)
            if (tb[i].w0 != kEmptyW0) h.table_entries++;
    }
    w.raw(&h, sizeof(h));
    if (e == cudaSuccess) e = w.dev(kSecNodes, c->d_nodes, sizeof(DNode) * c->S);
    if (e == cudaSuccess) e = w.dev(kSecLow, c->d_low, sizeof(double2) * c->S);
    if (e == cudaSuccess) e = w.dev(kSecIbox, c->d_ibox, sizeof(IBox) * c->S);
    if (e == cudaSuccess) e = w.dev(kSecSstack, c->d_sstack, sizeof(uint32_t) * c->S);
    if (e == cudaSuccess) e = w.dev(kSecGstack, c->d_gstack, sizeof(uint32_t) * c->G);
    if (e == cudaSuccess) e = w.dev(kSecGridCount, c->d_grid_count, sizeof(uint32_t) * ((size_t)c->G + 1));
    if (e == cudaSuccess) e = w.dev(kSecOrder, c->d_order, sizeof(uint32_t) * N);
    /* the table as runs, one per transfer chunk: a count, its slots, its
     * records; then a zero count */
    const uint64_t runs = (c->B + kTableChunk - 1) / kTableChunk;
    w.section(kSecTable, h.table_entries * (sizeof(unsigned long long) + sizeof(TRec)) + (runs + 1) * sizeof(uint64_t));
    for (uint64_t b = 0; b < c->B && e == cudaSuccess; b += kTableChunk) {
        const uint64_t n = std::min<uint64_t>(kTableChunk, c->B - b);
        tb.resize(n);
        e = cudaMemcpy(tb.data(), c->d_tab + b, sizeof(TRec) * n, cudaMemcpyDeviceToHost);
        slots.clear();
        recs.clear();
        for (uint64_t i = 0; i < n; ++i)
            if (tb[i].w0 != kEmptyW0) {
                slots.push_back(b + i);
                recs.push_back(tb[i]);
            }
        const uint64_t cntr = slots.size();
        w.raw(&cntr, sizeof(cntr));
        w.raw(slots.data(), sizeof(unsigned long long) * slots.size());
        w.raw(recs.data(), sizeof(TRec) * recs.size());
    }
    {
        const uint64_t zero = 0;
        w.raw(&zero, sizeof(zero));
    }
    /* the pending keys of the window */
    const uint64_t kv = h.counters.kv_count < c->kv_cap ? h.counters.kv_count : c->kv_cap;
    if (e == cudaSuccess) e = w.dev(kSecKeys, c->d_keys, sizeof(ulonglong2) * kv);
    if (e == cudaSuccess) e = w.dev(kSecKvBox, c->d_kvbox, sizeof(float4) * kv);
    if (e == cudaSuccess) e = w.dev(kSecSame, c->d_same, sizeof(uint32_t) * N);
    if (e == cudaSuccess) e = w.dev(kSecObox, c->d_obox, sizeof(uint4) * N);
    if (e == cudaSuccess) e = w.dev(kSecSids, c->d_sids, sizeof(uint16_t) * N);
    /* the last step's meetings, in log order */
    {
        const uint64_t m = std::min<uint64_t>(h.counters.meetings, c->log_cap);
        std::vector<glint_meeting> ms(m);
        const uint64_t b0 = h.counters.log_step_begin % c->log_cap;
        const uint64_t first = std::min<uint64_t>(m, c->log_cap - b0);
        if (e == cudaSuccess && first) e = cudaMemcpy(ms.data(), c->d_log + b0, sizeof(glint_meeting) * first, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && first < m)
            e = cudaMemcpy(ms.data() + first, c->d_log, sizeof(glint_meeting) * (m - first), cudaMemcpyDeviceToHost);
        w.section(kSecMeetings, sizeof(glint_meeting) * m);
        w.raw(ms.data(), sizeof(glint_meeting) * m);
    }
    /* the last flushed store */
    if (c->store_valid) {
        const uint64_t sk = c->store.kv_count + c->store.oversize_kv_count;
        if (e == cudaSuccess) e = w.dev(kSecStoreKeys, c->store_keys_ptr, sizeof(ulonglong2) * sk);
        if (e == cudaSuccess) e = w.dev(kSecStoreBoxes, c->store_boxes_ptr, sizeof(float4) * sk);
        if (e == cudaSuccess) e = w.dev(kSecCtfKeys, c->d_ctf_keys, c->store.key_bytes);
        if (e == cudaSuccess) e = w.dev(kSecSidsOut, c->d_sids_out, sizeof(uint16_t) * N);
        if (e == cudaSuccess) e = w.dev(kSecCtfs, c->d_ctfs, sizeof(glint_ctf_meta) * C);
        if (e == cudaSuccess) e = w.dev(kSecBitmaps, c->d_bitmaps, (size_t)C * 65536 / 8);
        if (e == cudaSuccess) e = w.dev(kSecObitmap, c->d_obitmap, 65536 / 8);
        w.section(kSecCtfCap, sizeof(uint32_t) * C);
        w.raw(c->store_ctf_cap.data(), sizeof(uint32_t) * C);
    }
    /* the blocks kept for queries */
    for (const StoreBlock &b : c->ctbs) {
        SnapBlock meta;
        std::memset(&meta, 0, sizeof(meta));
        meta.kv = b.kv;
        meta.o_count = b.o_count;
        meta.key_bytes = b.key_bytes;
        meta.end_time_min = b.end_time_min;
        meta.end_time_max = b.end_time_max;
        meta.C = b.C;
        meta.sid_count = b.sid_count;
        meta.oversize_oid_count = b.oversize_oid_count;
        std::memcpy(meta.o_times, b.o_times, sizeof(meta.o_times));
        std::memcpy(meta.rec_times, b.rec_times, sizeof(meta.rec_times));
        const uint32_t BC = b.C;
        w.section(kSecBlock, sizeof(meta));
        w.raw(&meta, sizeof(meta));
        if (e == cudaSuccess) e = w.dev(kSecCtfKeys, b.keys, b.key_bytes);
        if (e == cudaSuccess) e = w.dev(kSecCtfs, b.ctfs, sizeof(glint_ctf_meta) * BC);
        if (e == cudaSuccess) e = w.dev(kSecCtfCap, b.key_index, sizeof(unsigned long long) * BC);
        if (e == cudaSuccess) e = w.dev(kSecCtfCap, b.byte_index, sizeof(unsigned long long) * BC);
        if (e == cudaSuccess) e = w.dev(kSecSidsOut, b.sids, sizeof(uint16_t) * N);
        if (e == cudaSuccess) e = w.dev(kSecSame, b.first, sizeof(uint32_t) * N);
        if (e == cudaSuccess) e = w.dev(kSecSame, b.count, sizeof(uint32_t) * N);
        if (e == cudaSuccess) e = w.dev(kSecStoreKeys, b.okeys, sizeof(ulonglong2) * b.o_count);
        if (e == cudaSuccess) e = w.dev(kSecStoreBoxes, b.oboxes, sizeof(float4) * b.o_count);
        if (e == cudaSuccess) e = w.dev(kSecBitmaps, b.bitmaps, (size_t)BC * kBitBytes);
        if (e == cudaSuccess) e = w.dev(kSecObitmap, b.obitmap, kBitBytes);
    }
    const bool wrote = w.ok;
    if (fclose(w.f) != 0 || !wrote) {
        c->last_error = std::string("snapshot: write to ") + path + " failed";
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    if (e != cudaSuccess) return snap_fail(c, e);
    return GLINT_OK;
}

extern "C" glint_status glint_snapshot_load(const char *path, int device, glint_ctx **out) {
    if (!path || !out) return GLINT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    Reader r;
    r.f = fopen(path, "rb");
    if (!r.f) return GLINT_ERR_INVALID_ARGUMENT;
    SnapHeader h;
    r.raw(&h, sizeof(h));
    if (!r.ok || h.magic != kMagic || h.version != kVersion || h.header_bytes != sizeof(SnapHeader)) {
        fclose(r.f);
        return GLINT_ERR_INVALID_ARGUMENT;
    }
    glint_config cfg = h.cfg;
    if (device >= 0) cfg.device = (uint32_t)device;
    /* a context of the same sizes, created on points at one corner of the
     * map; its schema, table and windows are then replaced */
    std::vector<double> corner((size_t)cfg.num_objects * 2);
    for (uint32_t i = 0; i < cfg.num_objects; ++i) {
        corner[2 * i] = h.mbr.low[0];
        corner[2 * i + 1] = h.mbr.low[1];
    }
    glint_ctx *c = nullptr;
    glint_status st = glint_create(&cfg, &h.mbr, corner.data(), nullptr, &c);
    if (st != GLINT_OK) {
        fclose(r.f);
        return st;
    }
    cudaStream_t s = c->stream;
    cudaError_t e = cudaStreamSynchronize(s);
    const uint32_t N = c->N, C = c->cfg.CTF_count;
    if (e == cudaSuccess) e = r.dev(kSecNodes, c->d_nodes, sizeof(DNode) * c->S);
    if (e == cudaSuccess) e = r.dev(kSecLow, c->d_low, sizeof(double2) * c->S);
    if (e == cudaSuccess) e = r.dev(kSecIbox, c->d_ibox, sizeof(IBox) * c->S);
    if (e == cudaSuccess) e = r.dev(kSecSstack, c->d_sstack, sizeof(uint32_t) * c->S);
    if (e == cudaSuccess) e = r.dev(kSecGstack, c->d_gstack, sizeof(uint32_t) * c->G);
    if (e == cudaSuccess) e = r.dev(kSecGridCount, c->d_grid_count, sizeof(uint32_t) * ((size_t)c->G + 1));
    if (e == cudaSuccess) e = r.dev(kSecOrder, c->d_order, sizeof(uint32_t) * N);
    /* the table (empty after create); every occupied bucket is committed
     * between steps */
    uint64_t tbytes = 0;
    if (e == cudaSuccess && r.ok && r.section(kSecTable, tbytes)) {
        unsigned long long *d_slots = nullptr;
        TRec *d_recs = nullptr;
        e = cudaMalloc((void **)&d_slots, sizeof(unsigned long long) * kTableChunk);
        if (e == cudaSuccess) e = cudaMalloc((void **)&d_recs, sizeof(TRec) * kTableChunk);
        std::vector<unsigned long long> slots;
        std::vector<TRec> recs;
        uint64_t seen = 0;
        const uint64_t runs = (c->B + kTableChunk - 1) / kTableChunk;
        for (uint64_t run = 0; run <= runs; ++run) {
            uint64_t n = 0;
            r.raw(&n, sizeof(n));
            if (run == runs) {
                if (n != 0) r.ok = false; /* the terminating zero */
                break;
            }
            if (!r.ok || n > kTableChunk || e != cudaSuccess) {
                r.ok = false;
                break;
            }
            if (n == 0) continue;
            slots.resize(n);
            recs.resize(n);
            r.raw(slots.data(), sizeof(unsigned long long) * n);
            r.raw(recs.data(), sizeof(TRec) * n);
            if (!r.ok) break;
            e = cudaMemcpy(d_slots, slots.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(d_recs, recs.data(), sizeof(TRec) * n, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) {
                k_table_scatter<<<grid_for(n, 256), 256, 0, s>>>(c->d_tab, c->d_stamp, d_slots, d_recs, n, c->B);
                e = cudaStreamSynchronize(s);
            }
            seen += n;
        }
        if (seen != h.table_entries) r.ok = false;
        if (d_slots) cudaFree(d_slots);
        if (d_recs) cudaFree(d_recs);
    }
    /* the pending keys */
    const uint64_t kv = h.counters.kv_count < c->kv_cap ? h.counters.kv_count : c->kv_cap;
    if (e == cudaSuccess && r.ok) e = r.dev(kSecKeys, c->d_keys, sizeof(ulonglong2) * kv);
    if (e == cudaSuccess && r.ok) e = r.dev(kSecKvBox, c->d_kvbox, sizeof(float4) * kv);
    if (e == cudaSuccess && r.ok) e = r.dev(kSecSame, c->d_same, sizeof(uint32_t) * N);
    if (e == cudaSuccess && r.ok) e = r.dev(kSecObox, c->d_obox, sizeof(uint4) * N);
    if (e == cudaSuccess && r.ok) e = r.dev(kSecSids, c->d_sids, sizeof(uint16_t) * N);
    /* the last step's meetings, back at their log positions */
    uint64_t mbytes = 0;
    if (e == cudaSuccess && r.ok && r.section(kSecMeetings, mbytes) && mbytes % sizeof(glint_meeting) == 0) {
        const uint64_t m = mbytes / sizeof(glint_meeting);
        std::vector<glint_meeting> ms(m);
        r.raw(ms.data(), mbytes);
        const uint64_t b0 = h.counters.log_step_begin % c->log_cap;
        const uint64_t first = std::min<uint64_t>(m, c->log_cap - b0);
        if (r.ok && first) e = cudaMemcpy(c->d_log + b0, ms.data(), sizeof(glint_meeting) * first, cudaMemcpyHostToDevice);
        if (r.ok && e == cudaSuccess && first < m)
            e = cudaMemcpy(c->d_log, ms.data() + first, sizeof(glint_meeting) * (m - first), cudaMemcpyHostToDevice);
    }
    /* the last flushed store, in the buffers the next flush does not write */
    if (e == cudaSuccess && r.ok && h.store_valid) {
        const uint64_t sk = h.store.kv_count + h.store.oversize_kv_count;
        c->store_keys_ptr = c->d_keys2;
        c->store_boxes_ptr = c->d_kvbox2;
        c->store_kv = h.store.kv_count;
        e = r.dev(kSecStoreKeys, c->d_keys2, sizeof(ulonglong2) * sk);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecStoreBoxes, c->d_kvbox2, sizeof(float4) * sk);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecCtfKeys, c->d_ctf_keys, h.store.key_bytes);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecSidsOut, c->d_sids_out, sizeof(uint16_t) * N);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecCtfs, c->d_ctfs, sizeof(glint_ctf_meta) * C);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecBitmaps, c->d_bitmaps, (size_t)C * 65536 / 8);
        if (e == cudaSuccess && r.ok) e = r.dev(kSecObitmap, c->d_obitmap, 65536 / 8);
        uint64_t cb = 0;
        c->store_ctf_cap.assign(C, 0);
        if (e == cudaSuccess && r.ok && r.section(kSecCtfCap, cb) && cb == sizeof(uint32_t) * C)
            r.raw(c->store_ctf_cap.data(), cb);
        else
            r.ok = false;
        c->store = h.store;
        c->store_valid = r.ok;
    }
    /* the kept blocks */
    for (uint32_t k = 0; k < h.num_blocks && e == cudaSuccess && r.ok; ++k) {
        uint64_t mb = 0;
        SnapBlock meta;
        if (!r.section(kSecBlock, mb) || mb != sizeof(meta)) break;
        r.raw(&meta, sizeof(meta));
        StoreBlock b;
        b.kv = meta.kv;
        b.o_count = meta.o_count;
        b.key_bytes = meta.key_bytes;
        b.end_time_min = meta.end_time_min;
        b.end_time_max = meta.end_time_max;
        b.C = meta.C;
        b.sid_count = meta.sid_count;
        b.oversize_oid_count = meta.oversize_oid_count;
        std::memcpy(b.o_times, meta.o_times, sizeof(b.o_times));
        std::memcpy(b.rec_times, meta.rec_times, sizeof(b.rec_times));
        const uint32_t BC = b.C;
        e = r.dev_alloc(kSecCtfKeys, (void **)&b.keys, b.key_bytes);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecCtfs, (void **)&b.ctfs, sizeof(glint_ctf_meta) * BC);
        if (e == cudaSuccess && r.ok)
            e = r.dev_alloc(kSecCtfCap, (void **)&b.key_index, sizeof(unsigned long long) * BC);
        if (e == cudaSuccess && r.ok)
            e = r.dev_alloc(kSecCtfCap, (void **)&b.byte_index, sizeof(unsigned long long) * BC);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecSidsOut, (void **)&b.sids, sizeof(uint16_t) * N);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecSame, (void **)&b.first, sizeof(uint32_t) * N);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecSame, (void **)&b.count, sizeof(uint32_t) * N);
        if (e == cudaSuccess && r.ok)
            e = r.dev_alloc(kSecStoreKeys, (void **)&b.okeys, sizeof(ulonglong2) * b.o_count);
        if (e == cudaSuccess && r.ok)
            e = r.dev_alloc(kSecStoreBoxes, (void **)&b.oboxes, sizeof(float4) * b.o_count);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecBitmaps, (void **)&b.bitmaps, (size_t)BC * kBitBytes);
        if (e == cudaSuccess && r.ok) e = r.dev_alloc(kSecObitmap, (void **)&b.obitmap, kBitBytes);
        c->ctbs.push_back(b); /* freed with the context, complete or not */
    }
    const bool read_ok = r.ok;
    fclose(r.f);
    /* counters and host-side state */
    if (e == cudaSuccess && read_ok) {
        e = cudaMemcpy(c->d_cnt, &h.counters, sizeof(DevCounters), cudaMemcpyHostToDevice);
        *c->h_cnt = h.counters;
    }
    if (e != cudaSuccess || !read_ok) {
        glint_destroy(c);
        return e != cudaSuccess ? (e == cudaErrorMemoryAllocation ? GLINT_ERR_OUT_OF_MEMORY : GLINT_ERR_CUDA)
                                : GLINT_ERR_INVALID_ARGUMENT;
    }
    c->step_index = h.step_index;
    c->last_time = h.last_time;
    c->end_time_min = h.end_time_min;
    c->flushes = h.flushes;
    c->last_stats = h.last_stats;
    c->stats_valid = true;
    *out = c;
    return GLINT_OK;
}
