"""ctypes binding of libxg.so (the C ABI declared in include/xg.h).

The library is the product path: there is no CPU fallback.  If libxg.so is
missing or cannot be loaded, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxg.so")

XG_OK = 0
XG_ERR_CAPACITY = 3
STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "capacity exceeded",
    4: "cut requested on an uncut (sub-)simplex", 5: "unsupported cut topology",
    6: "unsupported element, order or term", 7: "non-finite weight or matrix entry",
    8: "no usable CUDA device", 9: "quadrilateral interface scaling factor above its bound",
}

# every symbol include/xg.h declares, checked by the CPU test suite
EXPORTS = [
    "xg_status_string", "xg_last_error", "xg_device_ok",
    "xg_mesh_create", "xg_mesh_destroy", "xg_mesh_info", "xg_mesh_facet_elements",
    "xg_space_create", "xg_space_create_l2", "xg_space_destroy", "xg_space_info", "xg_space_element_dofs",
    "xg_interpolate_p1_perturb", "xg_cutinfo_update", "xg_mesh_check",
    "xg_facets_with_neighbor_types", "xg_elements_with_neighbor_facets",
    "xg_cut_rules", "xg_base_rule_size", "xg_base_rule", "xg_integrate", "xg_integrate_noalloc", "xg_integrate_subdiv", "xg_subdiv_moments_tet",
    "xg_mesh_create_tensor", "xg_cut_rules_ex", "xg_quad_rule_capacity", "xg_integrate_ex", "xg_integrate_fields",
    "xg_integrate_mlset", "xg_cut_rules_mlset", "xg_mlset_rule_capacity", "xg_mlset_mark",
    "xg_iso_integrate_mesh", "xg_iso_deformation", "xg_integrate_bnd",
    "xg_mlset_form_create", "xg_mlset_form_assemble", "xg_form_create", "xg_form_destroy", "xg_form_set_defined_on", "xg_form_set_bnd_terms", "xg_form_set_coef_terms", "xg_form_set_deformation", "xg_form_capacity",
    "xg_quad_form_create", "xg_quad_form_destroy", "xg_quad_form_capacity", "xg_quad_form_assemble",
    "xg_form_assemble", "xg_form_check", "xg_form_stage_events", "xg_cutfem_step", "xg_cutfem_marking",
    "xg_space_create_st", "xg_space_info_st", "xg_cutinfo_update_st", "xg_st_cut_rules", "xg_st_form_create",
    "xg_st_cutfem_step", "xg_step_graph_create", "xg_step_graph_launch", "xg_step_graph_destroy",
    "xg_step_graph_kernel_count", "xg_form_autotune", "xg_autotune_table", "xg_iso_moments_tet", "xg_mlp_param_count", "xg_learned_points",
    "xg_mlp_create", "xg_mlp_destroy", "xg_mlp_get_params", "xg_mlp_set_params", "xg_mlp_forward", "xg_mlp_forward_tc", "xg_mlp_check",
    "xg_mlp_loss_grad", "xg_mlp_adam_step", "xg_learned_moments_tet", "xg_learned_moments_tet_ex", "xg_learned_features",
    "xg_cutinfo_update_bnd", "xg_mesh_boundary", "xg_cutinfo_nodes", "xg_elements_with_threshold",
    "xg_lform_create", "xg_lform_set_deformation", "xg_lform_destroy", "xg_lform_assemble", "xg_lform_check",
]


class XgError(RuntimeError):
    def __init__(self, status, where, msg=""):
        super().__init__("%s: %s%s" % (where, STATUS.get(status, "status %d" % status), (" (" + msg + ")") if msg else ""))
        self.status = status


class Term(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("domain", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("hpow", ctypes.c_int32),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("d_defined_on", ctypes.c_void_p),
    ]


class LTerm(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("domain", ctypes.c_int32), ("order", ctypes.c_int32),
                ("e", ctypes.c_int32 * 3), ("coef", ctypes.c_double), ("d_gf", ctypes.c_void_p),
                ("d_defined_on", ctypes.c_void_p), ("gf_space", ctypes.c_void_p)]


class MlTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("hpow", ctypes.c_int32),
        ("normal_lset", ctypes.c_int32),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("ntup", ctypes.c_int32),
        ("h_tuples", ctypes.c_void_p),
        ("d_defined_on", ctypes.c_void_p),
    ]


class BTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("domain", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("hpow", ctypes.c_int32),
        ("coef", ctypes.c_double),
        ("d_defined_on", ctypes.c_void_p),
    ]


class CTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("domain", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("hpow", ctypes.c_int32),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("e", ctypes.c_int32 * 3),
        ("gf_space", ctypes.c_void_p),
        ("d_gf", ctypes.c_void_p),
        ("d_defined_on", ctypes.c_void_p),
        ("d_deform", ctypes.c_void_p),
    ]


class FMono(ctypes.Structure):
    _fields_ = [
        ("coef", ctypes.c_double),
        ("e", ctypes.c_int32 * 3),
        ("f0", ctypes.c_int32),
        ("f1", ctypes.c_int32),
        ("d0", ctypes.c_int32),
        ("d1", ctypes.c_int32),
    ]


class StTerm(ctypes.Structure):
    _fields_ = [
        ("base", Term),
        ("tref", ctypes.c_double),
        ("bc", ctypes.c_double * 3),
        ("bs", ctypes.c_double * 3),
        ("omega", ctypes.c_double),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
    ]


class Csr(ctypes.Structure):
    _fields_ = [
        ("d_row_dof", ctypes.c_void_p),
        ("d_rowptr", ctypes.c_void_p),
        ("d_cols", ctypes.c_void_p),
        ("d_vals", ctypes.c_void_p),
        ("d_counts", ctypes.c_void_p),
        ("cap_rows", ctypes.c_int64),
        ("cap_nnz", ctypes.c_int64),
    ]


_lib = None


def load():
    """Loads libxg.so; raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libxg.so is not built (%s). Build it with `python -m ngsxfem_gb300.build` "
            "or __graft_entry__.build(); there is no CPU fallback." % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    sig = {
        "xg_status_string": (ctypes.c_char_p, [I]),
        "xg_last_error": (ctypes.c_char_p, []),
        "xg_device_ok": (I, [P]),
        "xg_mesh_create": (I, [I, ctypes.c_int32, P, ctypes.c_int32, P, P]),
        "xg_mesh_create_tensor": (I, [I, ctypes.c_int32, P, ctypes.c_int32, P, P]),
        "xg_mesh_destroy": (I, [P]),
        "xg_mesh_info": (I, [P, P]),
        "xg_mesh_facet_elements": (I, [P, P]),
        "xg_space_create": (I, [P, I, P]),
        "xg_space_create_l2": (I, [P, I, P]),
        "xg_space_destroy": (I, [P]),
        "xg_space_info": (I, [P, P]),
        "xg_space_element_dofs": (I, [P, P]),
        "xg_interpolate_p1_perturb": (I, [P, I64, D, P]),
        "xg_cutinfo_update": (I, [P, P, P, P, P, P]),
        "xg_mesh_check": (I, [P]),
        "xg_facets_with_neighbor_types": (I, [P, P, P, I, I, I, P, P]),
        "xg_elements_with_neighbor_facets": (I, [P, P, P, P]),
        "xg_cut_rules": (I, [P, P, P, ctypes.c_int32, I, I, ctypes.c_int32, P, P, P, P]),
        "xg_cut_rules_ex": (I, [P, P, P, ctypes.c_int32, I, I, I, ctypes.c_int32, P, P, P, P]),
        "xg_quad_rule_capacity": (I, [I, I, I]),
        "xg_base_rule_size": (I, [I, I]),
        "xg_base_rule": (I, [I, I, P, P, I]),
        "xg_integrate": (I, [P, P, I, I, I, I, I, P, P, P]),
        "xg_integrate_ex": (I, [P, P, I, I, I, I, I, I, P, P, P]),
        "xg_integrate_fields": (I, [P, P, I, I, I, P, P, I, P, P, P, P, P]),
        "xg_integrate_mlset": (I, [P, P, ctypes.c_int32, P, ctypes.c_int32, I, I, I, I, P, P, P]),
        "xg_cut_rules_mlset": (I, [P, P, ctypes.c_int32, P, ctypes.c_int32, P, ctypes.c_int32, I, ctypes.c_int32,
                                   P, P, P, P]),
        "xg_mlset_rule_capacity": (I, [I, ctypes.c_int32, ctypes.c_int32, I]),
        "xg_mlset_mark": (I, [P, P, ctypes.c_int32, P, ctypes.c_int32, I, P, P]),
        "xg_iso_integrate_mesh": (I, [P, P, I, I, ctypes.c_double, I, I, I, I, P, P, P]),
        "xg_iso_deformation": (I, [P, P, ctypes.c_double, P, P, P]),
        "xg_integrate_bnd": (I, [P, P, I, I, I, I, I, P, P, P]),
        "xg_integrate_noalloc": (I, [P, P, I, I, I, I, I, P, P, P]),
        "xg_integrate_subdiv": (I, [P, P, I, I, I, I, I, I, P, P, P]),
        "xg_subdiv_moments_tet": (I, [P, ctypes.c_int64, I, P, P, P]),
        "xg_mlset_form_create": (I, [P, I, P, I, P, I, I, P]),
        "xg_mlset_form_assemble": (I, [P, P, P, P]),
        "xg_form_create": (I, [P, P, ctypes.c_int32, I, P]),
        "xg_form_destroy": (I, [P]),
        "xg_form_set_defined_on": (I, [P, ctypes.c_int32, P]),
        "xg_form_set_bnd_terms": (I, [P, P, ctypes.c_int32]),
        "xg_form_set_coef_terms": (I, [P, P, ctypes.c_int32]),
        "xg_form_set_deformation": (I, [P, P]),
        "xg_quad_form_create": (I, [P, P, ctypes.c_int32, I, P]),
        "xg_quad_form_destroy": (I, [P]),
        "xg_quad_form_capacity": (I, [P, P]),
        "xg_quad_form_assemble": (I, [P, P, P, P]),
        "xg_form_capacity": (I, [P, P]),
        "xg_form_assemble": (I, [P, P, P, P, P]),
        "xg_form_check": (I, [P]),
        "xg_form_stage_events": (I, [P, P, I]),
        "xg_cutfem_step": (I, [P, P, P, P]),
        "xg_cutfem_marking": (I, [P, P, P, P, P]),
        "xg_step_graph_create": (I, [P, P, P, I, P]),
        "xg_step_graph_launch": (I, [P, P]),
        "xg_step_graph_destroy": (I, [P]),
        "xg_step_graph_kernel_count": (I, [P, P]),
        "xg_form_autotune": (I, [P, P, P, P]),
        "xg_autotune_table": (I64, [P, I64]),
        "xg_iso_moments_tet": (I, [P, I64, I, I, P, P, P]),
        "xg_mlp_param_count": (I, [P]),
        "xg_learned_points": (I, [P]),
        "xg_mlp_create": (I, [ctypes.c_uint64, P]),
        "xg_mlp_destroy": (I, [P]),
        "xg_mlp_get_params": (I, [P, P, P]),
        "xg_mlp_set_params": (I, [P, P, P]),
        "xg_mlp_forward": (I, [P, P, I64, P, P]),
        "xg_mlp_forward_tc": (I, [P, P, I64, P, P]),
        "xg_mlp_check": (I, [P]),
        "xg_mlp_loss_grad": (I, [P, P, P, P, I64, P, P, P]),
        "xg_mlp_adam_step": (I, [P, P, ctypes.c_float, I64, P]),
        "xg_learned_moments_tet": (I, [P, P, I64, D, P, P, P]),
        "xg_learned_moments_tet_ex": (I, [P, P, I64, D, I, P, P, P]),
        "xg_learned_features": (I, [P, I64, P, P]),
        "xg_cutinfo_update_bnd": (I, [P, P, P, P, P, P]),
        "xg_mesh_boundary": (I, [P, P, P]),
        "xg_cutinfo_nodes": (I, [P, P, P, P, P, P, P, P, P, P, P, P]),
        "xg_elements_with_threshold": (I, [P, I64, I, D, P, P]),
        "xg_lform_create": (I, [P, P, ctypes.c_int32, P]),
        "xg_lform_set_deformation": (I, [P, P]),
        "xg_lform_destroy": (I, [P]),
        "xg_lform_assemble": (I, [P, P, P, P, P]),
        "xg_lform_check": (I, [P]),
        "xg_space_create_st": (I, [P, I, I, P]),
        "xg_space_info_st": (I, [P, P]),
        "xg_cutinfo_update_st": (I, [P, P, I, P, P, P, P]),
        "xg_st_cut_rules": (I, [P, P, I, P, ctypes.c_int32, I, I, I, ctypes.c_int32, P, P, P, P]),
        "xg_st_form_create": (I, [P, I, I, P, ctypes.c_int32, I, P]),
        "xg_st_cutfem_step": (I, [P, P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status, where):
    if status != XG_OK:
        msg = load().xg_last_error()
        raise XgError(status, where, msg.decode() if msg else "")


def call(name, *args):
    check(getattr(load(), name)(*args), name)
