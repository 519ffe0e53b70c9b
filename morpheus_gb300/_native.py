"""ctypes binding of libmorpheus_gb300.so (the C ABI in include/*.h).

There is no CPU fallback: if the CUDA library is missing or no GPU is visible,
calls raise.  Loading the library itself needs no GPU (the symbol check in the
CPU test-suite relies on that).
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmorpheus_gb300.so")
_lib = None

u64 = ctypes.c_uint64
i32 = ctypes.c_int
sz = ctypes.c_size_t
vp = ctypes.c_void_p
u64p = ctypes.POINTER(ctypes.c_uint64)
u32p = ctypes.POINTER(ctypes.c_uint32)


class GbTranscript(ctypes.Structure):
    """gb_transcript: the fields of zk-torch-3's Transcript in C layout."""
    _fields_ = [("st", ctypes.c_uint64 * 8), ("inb", ctypes.c_uint64 * 4), ("outb", ctypes.c_uint64 * 4),
                ("nin", ctypes.c_uint32), ("nout", ctypes.c_uint32)]


class NativeError(RuntimeError):
    pass


# name -> (restype, argtypes)
SIGNATURES = {
    "goldilocks_cuda_init": (i32, []),
    "poseidon2_cuda_init": (i32, []),
    "cuda_malloc": (i32, [ctypes.POINTER(vp), sz]),
    "cuda_free": (i32, [vp]),
    "cuda_memcpy_htod": (i32, [vp, vp, sz]),
    "cuda_memcpy_dtoh": (i32, [vp, vp, sz]),
    "cuda_memcpy_dtod": (i32, [vp, vp, sz]),
    "cuda_device_synchronize": (i32, []),
    "cuda_get_last_error": (i32, []),
    "cuda_peek_at_last_error": (i32, []),
    "cuda_mem_get_info": (i32, [ctypes.POINTER(sz), ctypes.POINTER(sz)]),
    "cuda_pool_trim": (i32, [sz]),
    "cuda_set_device": (i32, [i32]),
    "cuda_get_device": (i32, [ctypes.POINTER(i32)]),
    "cuda_get_device_count": (i32, [ctypes.POINTER(i32)]),
    "cuda_get_device_name": (i32, [i32, ctypes.c_char_p, i32]),
    "gl_batch_add": (i32, [vp, vp, vp, i32]),
    "gl_batch_sub": (i32, [vp, vp, vp, i32]),
    "gl_batch_mul": (i32, [vp, vp, vp, i32]),
    "gl_batch_inverse": (i32, [vp, vp, i32]),
    "ext2_batch_add_ffi": (i32, [vp, vp, vp, i32]),
    "ext2_batch_sub_ffi": (i32, [vp, vp, vp, i32]),
    "ext2_batch_mul_ffi": (i32, [vp, vp, vp, i32]),
    "sumcheck_round_message_ffi": (i32, [vp, vp, i32, sz, sz, i32]),
    "sumcheck_fold_ffi": (i32, [vp, vp, u64, i32, sz, sz]),
    "sumcheck_round_message_ext2_ffi": (i32, [vp, vp, i32, sz, sz, i32]),
    "sumcheck_fold_ext2_ffi": (i32, [vp, vp, u64, u64, i32, sz, sz]),
    "monolith_cuda_init": (i32, []),
    "monolith_merkle_tree_gl_ffi": (i32, [vp, vp, i32]),
    "monolith_merkle_tree_ext2_ffi": (i32, [vp, vp, i32]),
    "monolith_permute_test_ffi": (i32, [vp, vp]),
    "challenger_state_size": (i32, []),
    "challenger_alloc_states": (i32, [ctypes.POINTER(vp), i32]),
    "challenger_init_states": (i32, [vp, i32]),
    "challenger_observe_ffi": (i32, [vp, vp, i32]),
    "challenger_observe_slice_ffi": (i32, [vp, vp, i32, i32]),
    "challenger_sample_ffi": (i32, [vp, vp, i32]),
    "challenger_sample_array_ffi": (i32, [vp, vp, i32, i32]),
    "challenger_sample_ext2_ffi": (i32, [vp, vp, i32]),
    "challenger_sample_ext5_ffi": (i32, [vp, vp, i32]),
    "challenger_observe_ext2_ffi": (i32, [vp, vp, i32]),
    "challenger_copy_state_to_host": (i32, [vp, vp]),
    "challenger_copy_state_to_device": (i32, [vp, vp]),
    "gb_set_coop_threshold": (sz, [sz]),
    "gb_get_coop_threshold": (sz, []),
    "gb_set_merkle_top_nodes": (sz, [sz]),
    "gb_get_merkle_top_nodes": (sz, []),
    "gb_prover_set_coop_threshold": (i32, [vp, sz]),
    "gb_prover_set_merkle_top_nodes": (i32, [vp, sz]),
    "gb_set_stream": (i32, [vp]),
    "gb_get_stream": (vp, []),
    "gb_last_error": (ctypes.c_char_p, []),
    "gb_device_sm_count": (i32, []),
    "gb_launch_count": (ctypes.c_ulonglong, []),
    "gb_mulmod_probe": (i32, [vp, i32, i32]),
    "gb_transcript_new": (None, [ctypes.POINTER(GbTranscript), ctypes.c_char_p]),
    "gb_transcript_append_u64": (None, [ctypes.POINTER(GbTranscript), ctypes.c_char_p, u64]),
    "gb_transcript_append_ext2": (None, [ctypes.POINTER(GbTranscript), ctypes.c_char_p, u64p]),
    "gb_transcript_challenge_ext2": (None, [ctypes.POINTER(GbTranscript), ctypes.c_char_p, u64p]),
    "gb_sumcheck_prove_ext2": (i32, [ctypes.POINTER(GbTranscript), i32, i32, vp, vp, vp, vp, vp, vp]),
    "gb_sumcheck_prove_ext2_polys": (i32, [ctypes.POINTER(GbTranscript), i32, i32, vp, vp, vp, vp, vp, vp]),
    "gb_sumcheck_prove_base": (i32, [ctypes.POINTER(GbTranscript), i32, i32, vp, vp, vp, vp, vp, vp]),
    "gb_sumcheck_round_workspace_words": (sz, []),
    "gb_sumcheck_fold_round_ext2": (i32, [vp, i32, sz, vp, sz, i32, sz, u64, u64, vp, vp]),
    "poseidon2_hash_batch_ffi": (i32, [vp, vp, i32]),
    "poseidon2_compress_batch_ffi": (i32, [vp, vp, vp, i32]),
    "poseidon2_merkle_layer_ffi": (i32, [vp, vp, i32]),
    "poseidon2_merkle_tree_gl_ffi": (i32, [vp, vp, i32]),
    "poseidon2_merkle_tree_ext2_ffi": (i32, [vp, vp, i32]),
    "eq_dp_all_ffi": (i32, [vp, vp, vp, i32, ctypes.POINTER(vp)]),
    "ext2_eq_dp_all_ffi": (i32, [vp, vp, vp, i32, ctypes.POINTER(vp)]),
    "basefold_bit_reverse_gl_ffi": (i32, [vp, i32]),
    "basefold_bit_reverse_ext2_ffi": (i32, [vp, i32]),
    "basefold_bhc_interpolate_ffi": (i32, [vp, vp, vp, i32]),
    "basefold_encode_ffi": (i32, [vp, vp, i32, i32]),
    "basefold_fold_gl_ffi": (i32, [vp, vp, u64, vp, i32]),
    "basefold_fold_mixed_ffi": (i32, [vp, vp, u64, u64, vp, i32]),
    "basefold_fold_ext2_ffi": (i32, [vp, vp, u64, u64, vp, i32]),
    "basefold_sumcheck_interp_gl_ffi": (i32, [vp, i32]),
    "basefold_sumcheck_interp_ext2_ffi": (i32, [vp, i32]),
    "basefold_sumcheck_product_gl_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32]),
    "basefold_sumcheck_product_mixed_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32]),
    "basefold_sumcheck_product_ext2_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32]),
    "basefold_sumcheck_eval_gl_ffi": (i32, [vp, u64, vp, i32]),
    "basefold_sumcheck_eval_mixed_ffi": (i32, [vp, u64, u64, vp, i32]),
    "basefold_sumcheck_eval_ext2_ffi": (i32, [vp, u64, u64, vp, i32]),
    "fused_sumcheck_round_ext2_ffi": (i32, [vp, vp, u64, u64, vp, vp, vp, vp, vp, i32, i32]),
    "basefold_dot_product_gl_ffi": (i32, [vp, vp, vp, i32, i32]),
    "basefold_dot_product_mixed_ffi": (i32, [vp, vp, vp, i32, i32]),
    "gb_basefold_table_create": (i32, [i32, i32, i32, u64, ctypes.POINTER(vp)]),
    "gb_basefold_table_destroy": (i32, [vp]),
    "gb_basefold_table_info": (i32, [vp, ctypes.POINTER(vp), vp]),
    "gb_basefold_commit": (i32, [vp, vp, i32, i32, ctypes.POINTER(vp), vp]),
    "gb_basefold_commitment_destroy": (i32, [vp]),
    "gb_basefold_commitment_info": (i32, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), vp]),
    "gb_basefold_proof_len": (sz, [i32, i32, i32]),
    "gb_basefold_open_ext2": (i32, [vp, vp, vp, ctypes.POINTER(GbTranscript), i32, vp]),
    "gb_basefold_batch_proof_len": (sz, [i32, i32, i32, i32]),
    "gb_basefold_batch_open_ext2": (i32, [vp, i32, vp, i32, vp, vp, vp, i32, vp, ctypes.POINTER(GbTranscript), i32,
                                          vp]),
    "gb_instance_proof_len": (sz, [i32, i32, i32]),
    "gb_instance_hbm_bytes": (sz, [i32, i32]),
    "gb_prove_instance": (i32, [vp, vp, i32, vp]),
    "gb_prover_create": (i32, [vp, vp, i32, i32, sz, ctypes.POINTER(vp)]),
    "gb_prover_submit": (i32, [vp, vp, ctypes.POINTER(ctypes.c_uint64)]),
    "gb_prover_wait": (i32, [vp, ctypes.c_uint64, vp]),
    "gb_prover_drain": (i32, [vp]),
    "gb_prover_destroy": (i32, [vp]),
    "gb_batch_prove": (i32, [vp, vp, i32, vp, i32, i32, sz]),
    "gb_batch_prove_lockstep": (i32, [vp, vp, i32, vp, i32, i32, sz]),
    "gb_lockstep_last_timing": (None, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gb_matmul_proof_len": (sz, [i32, i32, i32, i32]),
    "gb_matmul_hbm_bytes": (sz, [i32, i32, i32]),
    "gb_prove_matmul": (i32, [vp, vp, vp, i32, vp]),
    "gb_prover_set_ajtai_key": (i32, [vp, vp]),
    "gb_prover_submit_matmul": (i32, [vp, vp, ctypes.POINTER(ctypes.c_uint64)]),
    "almost_goldilocks_cuda_init": (i32, []),
    "agl_cuda_error_string": (ctypes.c_char_p, [i32]),
    "cuda_memset": (i32, [vp, i32, sz]),
    "cuda_sync_mine": (i32, []),
    "cuda_stream_create": (i32, [ctypes.POINTER(vp)]),
    "cuda_stream_destroy": (i32, [vp]),
    "cuda_stream_synchronize": (i32, [vp]),
    "cuda_memcpy_dtod_async": (i32, [vp, vp, sz, vp]),
    "cuda_memcpy_htod_async": (i32, [vp, vp, sz, vp]),
    "agl_cached_bytes": (sz, []),
    "agl_d2h_staged": (i32, [vp, vp, sz]),
    "agl_h2d_staged": (i32, [vp, vp, sz]),
    "agl_sumcheck_round_message_ffi": (i32, [vp, vp, i32, sz, sz, i32]),
    "agl_sumcheck_fold_ffi": (i32, [vp, vp, u64, i32, sz, sz]),
    "aext2_sumcheck_round_message_ffi": (i32, [vp, vp, i32, sz, sz, i32]),
    "aext2_sumcheck_fold_ffi": (i32, [vp, vp, u64, u64, i32, sz, sz]),
    "aext2_sumcheck_batched_round_message_ffi": (i32, [vp, vp, sz, sz, i32, i32]),
    "aext2_sumcheck_batched_fold_ffi": (i32, [vp, vp, u64, u64, sz, sz, i32]),
    "agl_eq_dp_all_ffi": (i32, [vp, vp, vp, i32, ctypes.POINTER(vp)]),
    "aext2_eq_dp_all_ffi": (i32, [vp, vp, vp, i32, ctypes.POINTER(vp)]),
    "aext2_eq_dp_all_stream_ffi": (i32, [vp, vp, vp, i32, ctypes.POINTER(vp), vp]),
    "aext2_eq_dp_all_batched_ffi": (i32, [vp, vp, vp, i32, i32, sz, ctypes.POINTER(vp), vp]),
    "ajtai_commit_wide_ffi": (i32, [vp, vp, u64, u64, i32, vp]),
    "ajtai_commit_wide_noalloc_ffi": (i32, [vp, vp, u64, u64, i32, vp]),
    "ajtai_materialize_m_ffi": (i32, [vp, vp, u64]),
    "ajtai_commit_ternary_premat_ffi": (i32, [vp, vp, vp, u64, i32, vp]),
    "ajtai_fold_witness_ffi": (i32, [vp, vp, vp, u64, i32, vp]),
    "ajtai_multifold_witness_ffi": (i32, [vp, vp, vp, i32, u64, u64]),
    "ajtai_multifold_mixed_witness_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32, u64, u64]),
    "ajtai_multifold_mixed_witness_tc_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32, u64]),
    "ajtai_multifold_mixed_witness_tc_fused_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32, u64]),
    "ajtai_split_witness_ffi": (i32, [vp, vp, vp, u64]),
    "ajtai_multifold_commitment_ffi": (i32, [vp, vp, i32, vp]),
    "ajtai_fold_commitment_ffi": (i32, [vp, vp, vp, vp]),
    "partial_eval_gl_ffi": (i32, [vp, vp, i32, i32]),
    "partial_eval_ext2_from_gl_ffi": (i32, [vp, vp, vp, i32, i32]),
    "bit_permute_gl_ffi": (i32, [vp, vp, vp, i32, i32]),
    "fused_permute_partial_eval_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32, i32, i32, i32]),
    "agl_partial_eval_ffi": (i32, [vp, vp, i32, i32]),
    "agl_partial_eval_ext2_from_base_ffi": (i32, [vp, vp, vp, i32, i32]),
    "agl_bit_permute_ffi": (i32, [vp, vp, vp, i32, i32]),
    "agl_fused_permute_partial_eval_ffi": (i32, [vp, vp, vp, vp, vp, i32, i32, i32, i32, i32]),
    "ajtai_commit_dense_batched_ffi": (i32, [vp, vp, u64, i32, i32, vp]),
    "ajtai_commit_dense_batched_at_ffi": (i32, [vp, vp, u64, i32, i32, u64, vp]),
    "ajtai_commit_ternary_ffi": (i32, [vp, vp, vp, u64, i32, vp]),
    "ajtai_commit_sparse_ffi": (i32, [vp, vp, u64, i32, vp]),
    "gb_ajtai_key_create": (i32, [vp, i32, i32, u64, ctypes.POINTER(vp)]),
    "gb_ajtai_key_destroy": (i32, [vp]),
    "gb_ajtai_key_info": (i32, [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(u64)]),
    "gb_ajtai_commit_u8_batched": (i32, [vp, vp, i32, vp]),
}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError(
                f"{LIB_PATH} is missing: build it with morpheus_gb300.build.build() "
                "(there is no CPU fallback for the prover kernels)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, what):
    if rc != 0:
        msg = lib().gb_last_error() or b""
        raise NativeError(f"{what} failed with code {rc}: {msg.decode(errors='replace')}")
