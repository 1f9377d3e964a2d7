/*
 * ref_gpu_layout.cpp -- prints the byte layout of the reference's workbench,
 * configuration, CTF and meeting_unit (tracing/workbench.h:62-383,
 * util/config.h:15-114, tracing/step_merge.h:58-90) as a header of offsets,
 * for oracle/ref_gpu_driver.cpp, which fills a device-resident workbench the
 * way cuda_create_device_bench does and runs the reference's own kernels.
 * TEST INFRASTRUCTURE: built and run by oracle/build_ref.sh where the
 * reference sources are; only numbers are emitted.
 */
#include <cstddef>
#include <cstdio>

#include "tracing/workbench.h"

#define EMIT(P, T, f) std::printf("#define RG_%s_%s %zu\n", P, #f, (size_t)offsetof(T, f))

int main() {
    std::printf("/* generated by oracle/ref_gpu_layout.cpp from the reference's headers */\n");
    std::printf("#define RG_WB_SIZE %zu\n", sizeof(workbench));
    EMIT("WB", workbench, config);
    EMIT("WB", workbench, cur_time);
    EMIT("WB", workbench, mbr);
    EMIT("WB", workbench, meeting_buckets);
    EMIT("WB", workbench, d_keys);
    EMIT("WB", workbench, d_ctf_keys);
    EMIT("WB", workbench, kv_count);
    EMIT("WB", workbench, dProbFalse);
    EMIT("WB", workbench, search_single);
    EMIT("WB", workbench, search_multi);
    EMIT("WB", workbench, search_multi_list);
    EMIT("WB", workbench, search_multi_length);
    EMIT("WB", workbench, search_multi_pid);
    EMIT("WB", workbench, multi_find_count);
    EMIT("WB", workbench, mid_xys);
    EMIT("WB", workbench, same_pid_count);
    EMIT("WB", workbench, d_sids);
    EMIT("WB", workbench, kv_boxs);
    EMIT("WB", workbench, o_boxs);
    EMIT("WB", workbench, oversize_oid_count);
    EMIT("WB", workbench, d_bitmaps);
    EMIT("WB", workbench, bit_count);
    EMIT("WB", workbench, bitmaps_size);
    EMIT("WB", workbench, d_oids);
    EMIT("WB", workbench, sid_count);
    EMIT("WB", workbench, d_CTF_capacity);
    EMIT("WB", workbench, d_ctfs);
    EMIT("WB", workbench, end_time_min);
    std::printf("#define RG_CFG_SIZE %zu\n", sizeof(configuration));
    EMIT("CFG", configuration, num_objects);
    EMIT("CFG", configuration, num_meeting_buckets);
    EMIT("CFG", configuration, min_meet_time);
    EMIT("CFG", configuration, max_meet_time);
    EMIT("CFG", configuration, kv_capacity);
    EMIT("CFG", configuration, CTF_count);
    EMIT("CFG", configuration, split_num);
    EMIT("CFG", configuration, search_multi_capacity);
    EMIT("CFG", configuration, search_single_capacity);
    std::printf("#define RG_CTF_SIZE %zu\n", sizeof(CTF));
    EMIT("CTF", CTF, ctf_mbr);
    EMIT("CTF", CTF, CTF_kv_capacity);
    EMIT("CTF", CTF, start_time_min);
    EMIT("CTF", CTF, start_time_max);
    EMIT("CTF", CTF, end_time_min);
    EMIT("CTF", CTF, end_time_max);
    EMIT("CTF", CTF, ctf_bitmap_size);
    EMIT("CTF", CTF, key_bit);
    EMIT("CTF", CTF, id_bit);
    EMIT("CTF", CTF, duration_bit);
    EMIT("CTF", CTF, end_bit);
    EMIT("CTF", CTF, low_x_bit);
    EMIT("CTF", CTF, low_y_bit);
    EMIT("CTF", CTF, edge_bit);
    EMIT("CTF", CTF, mbr_bit);
    EMIT("CTF", CTF, x_grid);
    EMIT("CTF", CTF, y_grid);
    std::printf("#define RG_MU_SIZE %zu\n", sizeof(meeting_unit));
    EMIT("MU", meeting_unit, key);
    EMIT("MU", meeting_unit, start);
    EMIT("MU", meeting_unit, end);
    EMIT("MU", meeting_unit, mbr);
    std::printf("#define RG_SIU_SIZE %zu\n", sizeof(search_info_unit));
    std::printf("#define RG_UINT_BOX_SIZE %zu\n", sizeof(uint_box));
    std::printf("#define RG_F_BOX_SIZE %zu\n", sizeof(f_box));
    std::printf("#define RG_BOX_SIZE %zu\n", sizeof(box));
    std::printf("#define RG_BLOCK_DIM %d\n", (int)BLOCK_DIM);
    std::printf("#define RG_BITMAP_EDGE %d\n", (int)DEFAULT_bitmap_edge);
    return 0;
}
