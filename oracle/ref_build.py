"""Builds the reference's own CUDA kernels for the GPU parity harness.

TEST INFRASTRUCTURE ONLY.  Run where the reference sources are, at
/root/reference; outputs go to oracle/_ref/ (git-ignored), which travels with
a copy of the repository to a machine without them.  Nothing here is copied
from the reference: its sources are compiled where they lie.

  * <prog>.cubin  — the reference program compiled for sm_103a with
                    `nvcc -cubin` (device code only; its host main is ignored).
                    YCSB/1/ycsb.cu and TPCC-allopt-final/tp.cu, as shipped;
                    and copies with constants of Predefine.h changed (each
                    compiled from a temporary copy outside the repository,
                    the way the reference's own sweep scripts rewrite those
                    lines, TPCC-allopt-final/tpcc_script.py:18-44):
                      tf50:   NEWORDER_PERCENT = 50 (32,768 NewOrders +
                              32,768 Payments);
                      tf_c3:  BATCH_SIZE = 1,048,576, NEWORDER_PERCENT = 50
                              (the TPC-C headline batch, W = 64);
                      y1_c2:  BATCH_SIZE = 1,048,576, YCSB_SIZE = 10,000,000,
                              16 ops of which 15 reads, uniform mode (the
                              YCSB high-contention scale; uniform mode drops
                              the shipped build's key-0 bypass, so every key
                              registers and is checked).
  * <prog>_layout.json — sizes and field offsets of the reference's buffer
                    structs and its launch constants, printed by a small host
                    program of ours that includes the reference's Predefine.h /
                    Datastructure.h (so the harness fills the buffers exactly
                    as the reference lays them out).
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# root of the reference project (read-only); the recipe builds nothing when absent
REF = os.path.join(os.environ.get("LTPG_REFERENCE_ROOT", "/root/reference"), "LTPG")
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")

PROGRAMS = {
    "y1": dict(dir="YCSB/1", main="ycsb.cu", layout=r'''
#include <cstdio>
#include <cstddef>
#include "Datastructure.h"
int main() {
  printf("{\"batch\": %u, \"table\": %llu, \"ops\": %u, \"reads\": %u, \"zipf\": %u,", BATCH_SIZE, YCSB_SIZE,
         YCSB_OP_SIZE, YCSB_READ_SIZE, DATA_DISTRIBUTION == ZIPFIAN ? 1u : 0u);
  printf("\"grids\": [%u, %u, %u], \"blocks\": [%u, %u, %u],", EXECUTE_GRID_SIZE, CHECK_GRID_SIZE,
         WRITEBACK_GRID_SIZE, EXECUTE_BLOCK_SIZE, CHECK_BLOCK_SIZE, WRITEBACK_BLOCK_SIZE);
  printf("\"set\": {\"size\": %zu, \"war\": %zu, \"raw\": %zu, \"waw\": %zu, \"commit\": %zu},",
         sizeof(YCSB_A_SET), offsetof(YCSB_A_SET, war), offsetof(YCSB_A_SET, raw), offsetof(YCSB_A_SET, waw),
         offsetof(YCSB_A_SET, COMMIT_AND_ABORT));
  printf("\"query\": {\"size\": %zu, \"loc_r\": %zu, \"loc_w\": %zu, \"tid\": %zu},", sizeof(YCSB_A_QUERY),
         offsetof(YCSB_A_QUERY, LOC_R), offsetof(YCSB_A_QUERY, LOC_W), offsetof(YCSB_A_QUERY, TID));
  printf("\"log\": {\"size\": %zu, \"ytd\": %zu},", sizeof(YCSB_LOG), offsetof(YCSB_LOG, YTD));
  printf("\"snapshot\": %zu, \"index\": %zu}\n", sizeof(YCSB_SNAPSHOT), sizeof(YCSB_INDEX));
}
''', kernels=["_Z14KERNEL_EXECUTEP10YCSB_A_SETP12YCSB_A_QUERYP8YCSB_LOGP13YCSB_SNAPSHOTP10YCSB_INDEX",
              "_Z12KERNEL_CHECKP10YCSB_A_SETP12YCSB_A_QUERYP8YCSB_LOGP13YCSB_SNAPSHOTP10YCSB_INDEX",
              "_Z16KERNEL_WRITEBACKP10YCSB_A_SETP12YCSB_A_QUERYP8YCSB_LOGP13YCSB_SNAPSHOTP10YCSB_INDEX"]),
    "tf": dict(dir="TPCC-allopt-final", main="tp.cu", layout=r'''
#include <cstdio>
#include <cstddef>
#include "Datastructure.h"
#define OFF(S, f) offsetof(S, f)
int main() {
  printf("{\"batch\": %u, \"warehouses\": %llu, \"neworder_cnt\": %u, \"payment_cnt\": %u,", BATCH_SIZE,
         WAREHOUSE_SIZE, NEWORDER_CNT, PAYMENT_CNT);
  printf("\"grids\": [%u, %u, %u], \"blocks\": [%u, %u, %u],", EXECUTE_GRID_SIZE, CHECK_GRID_SIZE,
         WRITEBACK_GRID_SIZE, EXECUTE_BLOCK_SIZE, CHECK_BLOCK_SIZE, WRITEBACK_BLOCK_SIZE);
  printf("\"neworder_set\": %zu, \"neworder_query\": %zu,", sizeof(NEWORDER_SET), sizeof(NEWORDER_QUERY));
  printf("\"neworder_counters\": {\"war\": %zu, \"raw\": %zu, \"waw\": %zu},", OFF(NEWORDER_SET, war),
         OFF(NEWORDER_SET, raw), OFF(NEWORDER_SET, waw));
  printf("\"neworder_fields\": {\"W_ID\": %zu, \"D_ID\": %zu, \"C_ID\": %zu, \"O_ID\": %zu, \"N_O_ID\": %zu, "
         "\"O_OL_CNT\": %zu, \"O_OL_ID\": %zu, \"OL_I_ID\": %zu, \"OL_SUPPLY_W_ID\": %zu, \"OL_QUANTITY\": %zu, "
         "\"TID\": %zu},", OFF(NEWORDER_QUERY, W_ID), OFF(NEWORDER_QUERY, D_ID), OFF(NEWORDER_QUERY, C_ID),
         OFF(NEWORDER_QUERY, O_ID), OFF(NEWORDER_QUERY, N_O_ID), OFF(NEWORDER_QUERY, O_OL_CNT),
         OFF(NEWORDER_QUERY, O_OL_ID), OFF(NEWORDER_QUERY, OL_I_ID), OFF(NEWORDER_QUERY, OL_SUPPLY_W_ID),
         OFF(NEWORDER_QUERY, OL_QUANTITY), OFF(NEWORDER_QUERY, TID));
  printf("\"payment_set\": {\"size\": %zu, \"war\": %zu, \"raw\": %zu, \"waw\": %zu},", sizeof(PAYMENT_SET),
         OFF(PAYMENT_SET, war), OFF(PAYMENT_SET, raw), OFF(PAYMENT_SET, waw));
  printf("\"payment_query\": {\"size\": %zu, \"W_ID\": %zu, \"D_ID\": %zu, \"C_ID\": %zu, \"C_LAST\": %zu, "
         "\"isName\": %zu, \"C_D_ID\": %zu, \"C_W_ID\": %zu, \"H_AMOUNT\": %zu, \"H_ID\": %zu, \"TID\": %zu},",
         sizeof(PAYMENT_QUERY), OFF(PAYMENT_QUERY, W_ID), OFF(PAYMENT_QUERY, D_ID), OFF(PAYMENT_QUERY, C_ID),
         OFF(PAYMENT_QUERY, C_LAST), OFF(PAYMENT_QUERY, isName), OFF(PAYMENT_QUERY, C_D_ID),
         OFF(PAYMENT_QUERY, C_W_ID), OFF(PAYMENT_QUERY, H_AMOUNT), OFF(PAYMENT_QUERY, H_ID), OFF(PAYMENT_QUERY, TID));
  printf("\"log\": {\"size\": %zu, \"w_ytd\": %zu},", sizeof(LOG), OFF(LOG, W_YTD));
  printf("\"customer_size\": %llu, \"cust_snapshot\": %zu, \"name_index\": %zu,", CUSTOMER_SIZE,
         OFF(SNAPSHOT, customer_snapshot), OFF(INDEX, customer_name_index));
  printf("\"cid_grid\": %u, \"cid_block\": %u,", GRID_SIZE, BLOCK_SIZE);
  printf("\"snapshot\": %zu, \"index\": %zu}\n", sizeof(SNAPSHOT), sizeof(INDEX));
}
''', cid_kernel="_Z10KERNEL_CIDP11PAYMENT_SETP13PAYMENT_QUERYP3LOGP8SNAPSHOTP5INDEX",
        kernels=["_Z14KERNEL_EXECUTEP12NEWORDER_SETP11PAYMENT_SETP14NEWORDER_QUERYP13PAYMENT_QUERYP3LOGP8SNAPSHOTP5INDEX",
              "_Z12KERNEL_CHECKP12NEWORDER_SETP11PAYMENT_SETP14NEWORDER_QUERYP13PAYMENT_QUERYP3LOGP8SNAPSHOTP5INDEX",
              "_Z16KERNEL_WRITEBACKP12NEWORDER_SETP11PAYMENT_SETP14NEWORDER_QUERYP13PAYMENT_QUERYP3LOGP8SNAPSHOTP5INDEX"]),
}
# Copies with other constants: the shipped sources copied to a temporary
# directory outside the repository, lines of Predefine.h (consts, so not
# settable by -D) changed, compiled there.  Each patch must match once.
def _const(name, typ, old, new):
    return ("Predefine.h", rf"{name}\s*=\s*\({typ}\){old};", f"{name} =({typ}){new};")


PROGRAMS["tf50"] = dict(PROGRAMS["tf"], patches=[_const("NEWORDER_PERCENT", "unsigned int", 0, 50)])
PROGRAMS["tf_c3"] = dict(PROGRAMS["tf"], patches=[_const("BATCH_SIZE", "unsigned int", 65536, 1048576),
                                                  _const("NEWORDER_PERCENT", "unsigned int", 0, 50)])
PROGRAMS["y1_c2"] = dict(PROGRAMS["y1"], patches=[
    _const("BATCH_SIZE", "unsigned int", 10000, 1048576),
    _const("YCSB_SIZE", "unsigned long long", 1000000, 10000000),
    _const("YCSB_OP_SIZE", "unsigned int", 10, 16),
    _const("YCSB_READ_SIZE", "unsigned int", 9, 15),
    _const("DATA_DISTRIBUTION", "unsigned int", "ZIPFIAN", "UNIFORM")])
LAYOUT_VERSION = 2  # neworder_counters / neworder_fields


def available():
    return os.path.isdir(REF)


def build(force=False):
    """Compiles the cubins and layouts if the reference sources are present."""
    if not available():
        return False
    os.makedirs(OUT, exist_ok=True)
    for name, p in PROGRAMS.items():
        src_dir = os.path.join(REF, p["dir"])
        tmp = None
        if "patches" in p:
            tmp = tempfile.mkdtemp(prefix="ltpg_ref_")
            shutil.copytree(src_dir, os.path.join(tmp, "src"))
            src_dir = os.path.join(tmp, "src")
            for fname, pattern, repl in p["patches"]:
                path = os.path.join(src_dir, fname)
                text, n = re.subn(pattern, repl, open(path).read())
                if n != 1:
                    raise RuntimeError(f"{name}: patch {pattern!r} of {fname} matched {n} times")
                open(path, "w").write(text)
        try:
            _build_one(name, p, src_dir, force)
        finally:
            if tmp:
                shutil.rmtree(tmp, ignore_errors=True)
    return True


def _build_one(name, p, src_dir, force):
    cubin = os.path.join(OUT, f"{name}.cubin")
    layout = os.path.join(OUT, f"{name}_layout.json")
    if force or not os.path.exists(cubin):
        subprocess.run([NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-w", "-o", cubin, os.path.join(src_dir, p["main"])], check=True, capture_output=True)
    stale = os.path.exists(layout) and json.load(open(layout)).get("layout_version", 1) < LAYOUT_VERSION
    if force or stale or not os.path.exists(layout):
        cpp = os.path.join(OUT, f"{name}_layout.cpp")
        exe = os.path.join(OUT, f"{name}_layout")
        with open(cpp, "w") as f:
            f.write(p["layout"])
        subprocess.run(["g++", "-std=c++17", "-w", "-I" + src_dir, cpp, "-o", exe], check=True,
                       capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
        data = json.loads(out)
        data["kernels"] = p["kernels"]
        data["layout_version"] = LAYOUT_VERSION
        if "cid_kernel" in p:
            data["cid_kernel"] = p["cid_kernel"]
        with open(layout, "w") as f:
            json.dump(data, f, indent=1)
        os.remove(exe)
        os.remove(cpp)


if __name__ == "__main__":
    print("built" if build(force="--force" in sys.argv) else "reference sources not present")
