"""ctypes signatures of the sparse-DP, completion-table, batching and tree-DP entry points."""
import ctypes as c

vp, u64, i64, ci = c.c_void_p, c.c_uint64, c.c_int64, c.c_int

# the probe callback of tg_search: (m, zh, zl, lg, R, out, ctx) -> 0
PROBE_FN = c.CFUNCTYPE(ci, i64, c.POINTER(c.c_uint64), c.POINTER(c.c_uint64), c.POINTER(c.c_uint64),
                       c.POINTER(c.c_int32), c.POINTER(c.c_int32), vp)

SIGNATURES = {
    "tg_sp_clear": (ci, [vp, u64, vp]),
    "tg_sp_step": (ci, [vp, u64, vp, ci, vp, ci, vp, u64, vp, u64, u64, u64, u64, ci, ci, ci, ci, ci, ci, ci,
                        vp, vp, i64, u64, vp, vp]),
    "tg_sp_build": (ci, [vp, u64, vp, ci, ci, vp, vp, vp]),
    "tg_sp_join": (ci, [vp, u64, vp, ci, u64, vp, vp]),
    "tg_sp_lookup": (ci, [vp, ci, vp, u64, vp, vp]),
    "tg_sp_hist": (ci, [vp, u64, vp, vp]),
    "tg_sp_walk_scratch_bytes": (i64, [u64]),
    "tg_rank_profile": (ci, [ci, ci, vp, vp, vp, vp]),
    "tg_make_plan": (ci, [ci, ci, ci, vp, vp, vp, i64, vp, vp, vp]),
    "tg_sp_bound_data": (ci, [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp, ci, ci, ci, vp, vp, vp, vp]),
    "tg_sp_walk": (ci, [ci, vp, vp, vp, ci, ci, vp, u64, vp, ci, vp, u64, vp, u64, vp, vp, vp, vp, vp]),
    "tg_tab_create": (vp, [ci, ci, c.POINTER(ci)]),
    "tg_tab_free": (None, [vp]),
    "tg_tab_count": (i64, [vp]),
    "tg_tab_slots_log2": (i64, [vp]),
    "tg_tab_build": (ci, [vp, ci, vp, vp, vp, ci]),
    "tg_tab_lookup_dev": (ci, [vp, u64, vp, vp, vp, vp, vp, vp]),
    "tg_batch_create": (vp, [ci, vp, vp, c.POINTER(ci)]),
    "tg_batch_info": (ci, [vp, vp, ci]),
    "tg_batch_run": (ci, [vp, vp, ci, ci, vp, vp]),
    "tg_batch_free": (None, [vp]),
    "tg_server_create": (vp, [vp, u64, ci, i64, ci, ci, c.POINTER(ci)]),
    "tg_server_submit": (ci, [vp, vp, i64]),
    "tg_server_submit_plan": (ci, [vp, vp]),
    "tg_server_poll": (ci, [vp, vp, vp, ci]),
    "tg_server_stop": (ci, [vp]),
    "tg_server_free": (None, [vp]),
    "tg_search": (ci, [ci, ci, ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, ci, ci, ci, i64, PROBE_FN, vp,
                       vp, vp, ci, ci, c.c_double, vp, vp, vp]),
    "tree_join_u8": (ci, [vp, vp, vp, vp, vp, c.c_uint, c.c_uint, u64, u64, u64]),
    "tree_join_u16": (ci, [vp, vp, vp, vp, vp, c.c_uint, c.c_uint, u64, u64, u64]),
    "tree_join_u32": (ci, [vp, vp, vp, vp, vp, c.c_uint, c.c_uint, u64, u64, u64]),
    "tree_join_u64": (ci, [vp, vp, vp, vp, vp, c.c_uint, c.c_uint, u64, u64, u64]),
    "tree_move": (ci, [vp, vp, c.c_size_t]),
    "tg_tree_plan": (vp, [vp, i64, vp, i64, vp, i64, vp, i64, vp, i64, i64, i64, i64, i64, ci, c.POINTER(ci)]),
    "tg_tree_plan_info": (ci, [vp, vp, ci]),
    "tg_tree_run": (ci, [vp, vp, vp, c.c_uint32, c.POINTER(c.c_uint32), vp]),
    "tg_tree_plan_free": (None, [vp]),
}
