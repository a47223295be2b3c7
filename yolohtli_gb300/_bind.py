"""ctypes signatures of every function exported by libyolohtli_gb300.so
(include/yolohtli.h)."""
import ctypes as C

from . import _abi as A

_P = C.POINTER
_v = C.c_void_p
_i = C.c_int
_d = C.c_double
_f = C.c_float

SIGNATURES = {
    # parameter helpers
    "yh_param_defaults": (_i, [_P(A.ParamVar), _i, _i]),
    "yh_param_derive": (_i, [_P(A.ParamVar)]),
    "yh_fk_defaults": (_i, [_P(A.FKParams)]),
    "yh_status_string": (C.c_char_p, [_i]),
    "yh_version": (C.c_char_p, []),
    "yh_sizeof": (C.c_size_t, [C.c_char_p]),
    # stateless operators
    "yh_reaction_diffusion": (_i, [_P(A.ParamVar), _i, _P(A.FKParams), A.Fields,
                                   A.Fields, A.Fields, _v, _v]),
    "yh_spiral_tip": (_i, [_P(A.ParamVar), _v, _v, _d, _v, _v, _i, _v, _v]),
    "yh_pick_centre": (_i, [_v, _v, _i, _v, _v]),
    "yh_filament_mark": (_i, [_P(A.ParamVar), _v, _v, _v, _v]),
    "yh_contour": (_i, [_P(A.ParamVar), _v, _v, _v, _i, _f, _v, _v, _i, _v,
                        _v]),
    "yh_space_apd": (_i, [_P(A.ParamVar), _i, _v, _v, A.ApdFields, _v, _i,
                          _v]),
    "yh_phase_integrals_workspace": (C.c_size_t, [_i, _i]),
    "yh_phase_integrals": (_i, [_P(A.ParamVar), _i, A.Fields, A.Fields,
                                A.Fields, A.Fields, A.Fields, _v, _v, _v, _v,
                                _v, _v]),
    "yh_phase_integrals_noalloc": (_i, [_P(A.ParamVar), _i, A.Fields,
                                        A.Fields, A.Fields, A.Fields,
                                        A.Fields, _v, _v, _v, _v, _v]),
    "yh_phase_integrals_noalloc_limit": (C.c_size_t, []),
    "yh_template_slices": (_i, [_P(A.ParamVar), _i, A.Fields, A.Fields,
                                A.Fields, A.Fields, _v]),
    "yh_comoving_field": (_i, [_P(A.ParamVar), _v, _v, _v, _v, _v, _i, _v]),
    "yh_advect_bfecc": (_i, [_P(A.ParamVar), _i, A.Fields, A.Fields, _v, _v,
                             _v, A.Fields, A.Fields, _v]),
    "yh_advect_bfecc_3pass": (_i, [_P(A.ParamVar), _i, A.Fields, A.Fields, _v, _v,
                                   _v, A.Fields, A.Fields, _v]),
    "yh_sym_advance": (_i, [_P(A.ParamVar), _v, _v]),
    "yh_stimulate_box": (_i, [_P(A.ParamVar), _v, _v, _i, _i, _i, _i, _f, _v]),
    "yh_reaction_diffusion_f64": (_i, [_P(A.ParamVar), _i, _P(A.FKParams),
                                       A.Fields64, A.Fields64, A.Fields64, _v,
                                       _v]),
    "yh_spiral_tip_f64": (_i, [_P(A.ParamVar), _v, _v, _d, _v, _v, _i, _v, _v]),
    "yh_stimulate_box_f64": (_i, [_P(A.ParamVar), _v, _v, _i, _i, _i, _i, _d,
                                  _v]),
    # solver handle
    "yh_create": (_i, [_P(A.ParamVar), _i, _P(A.FKParams), _v, _v, _P(_v)]),
    "yh_destroy": (_i, [_v]),
    "yh_synchronize": (_i, [_v]),
    "yh_set_state": (_i, [_v, _v, _v, _v]),
    "yh_get_state": (_i, [_v, _v, _v, _v]),
    "yh_state_device": (_i, [_v, _P(A.Fields)]),
    "yh_set_time_block": (_i, [_v, _i]),
    "yh_get_time_block": (_i, [_v, _P(_i)]),
    "yh_set_engine": (_i, [_v, _i, _i]),
    "yh_get_engine": (_i, [_v, _P(_i), _P(_i)]),
    "yh_autotune": (_i, [_v, _i, _P(_i), _P(_i)]),
    "yh_run": (_i, [_v, _i, _P(A.Stim), _i]),
    "yh_track_tips": (_i, [_v]),
    "yh_get_tips": (_i, [_v, _P(A.Tip), _i, _P(_i)]),
    "yh_sr_begin": (_i, [_v, _i, _v, _v, _v]),
    "yh_sr_step": (_i, [_v, _i]),
    "yh_sr_enqueue": (_i, [_v, _i]),
    "yh_sr_status": (_i, [_v]),
    "yh_get_sym": (_i, [_v, _P(A.SymState)]),
    "yh_get_step": (_i, [_v, _P(_i)]),
    "yh_set_step": (_i, [_v, _i]),
    "yh_get_launch_count": (_i, [_v, _P(C.c_longlong)]),
    "yh_check_finite": (_i, [_v, _P(C.c_longlong)]),
    "yh_save_checkpoint": (_i, [_v, C.c_char_p]),
    "yh_load_checkpoint": (_i, [_v, C.c_char_p]),
    "yh_checkpoint_same_problem": (_i, [_P(A.ParamVar), _i, _P(A.FKParams),
                                        _P(A.ParamVar), _i, _P(A.FKParams)]),
    # batched solver
    "yh_batch_create": (_i, [_i, _P(A.ParamVar), _P(A.FKParams), _P(_v), _v,
                             _P(_v)]),
    "yh_batch_destroy": (_i, [_v]),
    "yh_batch_synchronize": (_i, [_v]),
    "yh_batch_set_state": (_i, [_v, _i, _v, _v, _v]),
    "yh_batch_get_state": (_i, [_v, _i, _v, _v, _v]),
    "yh_batch_state_device": (_i, [_v, _i, _P(A.Fields)]),
    "yh_batch_run": (_i, [_v, _i, _P(A.BatchStim), _i]),
    "yh_batch_run_host": (_i, [_v, _i, _P(A.BatchStim), _i, _P(_v), _P(_v),
                               _P(_v), _P(_v), _P(_v), _P(_v)]),
    "yh_batch_set_schedule": (_i, [_v, C.c_longlong, _i]),
    "yh_batch_autotune": (_i, [_v, _i, _P(C.c_longlong), _P(_i), _P(_i)]),
    "yh_batch_set_depth": (_i, [_v, _i]),
    "yh_batch_set_wave": (_i, [_v, _i, _i]),
    "yh_batch_get_wave": (_i, [_v, _P(_i), _P(_i), _P(_i)]),
    "yh_batch_get_step": (_i, [_v, _P(_i)]),
    "yh_batch_set_step": (_i, [_v, _i]),
    "yh_batch_get_launch_count": (_i, [_v, _P(C.c_longlong)]),
    "yh_selftest_resident_timeout": (_i, [_P(_i), _P(_i)]),
    # adjoint
    "yh_adjoint_create": (_i, [_P(A.ParamVar), _P(A.FKParams), _i, _i, _i, _i,
                               _i, _d, _v, _P(_v)]),
    "yh_adjoint_create_batch": (_i, [_P(A.ParamVar), _P(A.FKParams), _i, _i, _i,
                                     _i, _i, _i, C.c_double, _v, _P(_v)]),
    "yh_adjoint_batch": (_i, [_v, _P(_i)]),
    "yh_adjoint_destroy": (_i, [_v]),
    "yh_adjoint_probes": (_i, [_v, _P(_i), _P(_i), _P(_i)]),
    "yh_adjoint_set_target": (_i, [_v, _v]),
    "yh_adjoint_record": (_i, [_v, _v, _v, _v, _v, _v]),
    "yh_adjoint_run": (_i, [_v, _v, _v, _v, _v, _P(_d), _v]),
    "yh_adjoint_run_fk": (_i, [_v, _v, _v, _v, _v, _P(_d), _v, _P(A.FKParams)]),
    "yh_adjoint_set_fk": (_i, [_v, _P(A.FKParams)]),
    # the reference's interchange files
    "yh_write_param_csv": (_i, [C.c_char_p, _P(A.ParamVar), C.c_char_p,
                                C.c_char_p]),
    "yh_read_param_csv": (_i, [C.c_char_p, _P(A.ParamVar)]),
    "yh_write_raw_data": (_i, [C.c_char_p, _P(A.ParamVar), _v, _v]),
    "yh_read_raw_data": (_i, [C.c_char_p, _P(A.ParamVar), _v, _v]),
    "yh_write_raw_window": (_i, [C.c_char_p, _P(A.ParamVar), _v, _v]),
    "yh_write_tips": (_i, [C.c_char_p, C.c_char_p, _P(A.Tip), _i, _i]),
    "yh_write_sym_list": (_i, [C.c_char_p, _v, _v, _i]),
    # this library's binary checkpoint
    "yh_write_checkpoint": (_i, [C.c_char_p, _P(A.ParamVar), _i,
                                 _P(A.FKParams), _v, C.c_longlong, _v, _v,
                                 _v]),
    "yh_read_checkpoint_header": (_i, [C.c_char_p, _P(A.CheckpointHeader)]),
    "yh_read_checkpoint": (_i, [C.c_char_p, _P(A.ParamVar), _P(_i),
                                _P(A.FKParams), _v, _P(C.c_longlong), _v, _v,
                                _v]),
}


def declare(lib):
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
