// gen_state.h — the generator handle, shared by the host generator (gen.cpp)
// and the device generator (gen_dev.cu).
#pragma once
#include <vector>

#include "gen.h"

struct ltpg_gen_dev;  // device copy of the TPC-C generator state (gen_dev.cu)

struct ltpg_gen {
    int kind = 0;
    ltpg_ycsb_params y{};
    ltpg_tpcc_params c{};
    ltpg::gen::Zipf zipf;
    // TPC-C per-warehouse counters (TF/Query.h:54-88,157-166).
    std::vector<uint32_t> o_id, no_id, ol_id, h_id;
    // By-name Payments: C_LAST of every customer of the loaded image and its
    // rank among the customers of its district with that name, in C_ID order.
    std::vector<uint16_t> cust_name;
    std::vector<uint8_t> cust_rank;
    // OrderStatus / Delivery: the orders this generator made, per warehouse
    // (indexed by O_ID): customer, district, first OL_ID, line count; how many
    // were made and delivered.
    std::vector<uint16_t> o_cust;
    std::vector<uint8_t> o_dist, o_cnt;
    std::vector<uint32_t> o_ol;
    std::vector<uint64_t> made, delivered;
    uint64_t next_batch = 0, txn_base = 0;
    // Set by the first TPC-C batch made on the device: the counters and the
    // order memory then live there, and host batches are refused.
    bool dev_bound = false;
    ltpg_gen_dev *dev = nullptr;
};

// Frees the device state of g (gen_dev.cu).
void gen_dev_free(ltpg_gen *g);
// The sampler's power tables, filled once (gen.cpp).
const ltpg::gen::FixTables &host_fix_tables();
