"""ctypes mirror of include/sem2d_gpu.h and include/sem2d_host.h.

The field order here must match the C headers exactly; tests check the
structure sizes against the compiled library (``sem2d_abi_sizes``).
"""
import ctypes as C

c_int, c_double, c_char = C.c_int, C.c_double, C.c_char
P_int = C.POINTER(C.c_int)
P_double = C.POINTER(C.c_double)

# status codes (sem2d_gpu.h)
SEM2D_OK = 0
SEM2D_E_ARG = -1
SEM2D_E_CUDA = -2
SEM2D_E_UNSUPPORTED = -3
SEM2D_E_NR = -4
SEM2D_E_NAN = -5
SEM2D_E_STATE = -6
SEM2D_E_NOMEM = -7
SEM2D_E_TIMEOUT = -8

TIME_LEAPFROG = 0
TIME_NEWMARK = 1
TIME_HHT = 2
FRICTION_SWF = 1
FRICTION_RSF = 2
FRICTION_TWF = 3
PRECISION_FP64 = 0
PRECISION_MIXED = 1

STF_NONE = 0
STF_RICKER = 1
STF_TAB = 3
STF_HARMONIC = 4
STF_BRUNE = 5
STF_GAUSSIAN = 6
STF_USER = 7
STF_KINDS = {"RICKER": STF_RICKER, "TAB": STF_TAB, "HARMONIC": STF_HARMONIC,
             "BRUNE": STF_BRUNE, "GAUSSIAN": STF_GAUSSIAN, "USER": STF_USER}

WAVE_NONE = 0
WAVE_P = 1
WAVE_S = 2

BC_ABSORB = 1
BC_DYNFLT = 2
BC_DIRNEU = 3
BC_PERIOD = 4

MAX_DOMAINS = 64
MAX_MATS = 64
MAX_BCS = 16
MAX_LAYERS = 32

# per-node fault inputs (enum in sem2d_host.h)
FP_NAMES = ["Tt", "Tn", "Sxx", "Sxy", "Sxz", "Syz", "Szz", "cohesion", "V",
            "swf_dc", "swf_mus", "swf_mud", "swf_p", "swf_alpha",
            "rsf_dc", "rsf_mus", "rsf_a", "rsf_b", "rsf_vstar", "rsf_theta", "rsf_vc"]
FP_INDEX = {n: i for i, n in enumerate(FP_NAMES)}
FP_NPARAM = len(FP_NAMES)
# defaults of the reference's namelists (bc_dynflt.f90:105-140,
# bc_dynflt_swf.f90:71-82, bc_dynflt_rsf.f90:76-92)
FP_DEFAULTS = {"Tt": 0.0, "Tn": 0.0, "Sxx": 0.0, "Sxy": 0.0, "Sxz": 0.0, "Syz": 0.0,
               "Szz": 0.0, "cohesion": 0.0, "V": 1e-12,
               "swf_dc": 0.5, "swf_mus": 0.6, "swf_mud": 0.5, "swf_p": 3.0, "swf_alpha": 0.0,
               "rsf_dc": 0.5, "rsf_mus": 0.6, "rsf_a": 0.01, "rsf_b": 0.02, "rsf_vstar": 1.0,
               "rsf_theta": 0.0, "rsf_vc": 1e-6}


class Stf(C.Structure):
    """sem2d_stf: a source time function (STF_get, stf_gen.f90:99-121)."""
    _fields_ = [("kind", c_int), ("ntab", c_int),
                ("f0", c_double), ("onset", c_double), ("ampli", c_double),
                ("par1", c_double), ("par2", c_double),
                ("tab_t", P_double), ("tab_v", P_double)]


P_Stf = C.POINTER(Stf)


class ProblemDesc(C.Structure):
    _fields_ = [
        ("ngll", c_int), ("ndof", c_int), ("nelem", c_int), ("npoin", c_int),
        ("ibool", P_int), ("coord", P_double), ("hprime", P_double), ("wgll", P_double),
        ("Kx", P_double), ("Kz", P_double), ("la", P_double), ("mu", P_double), ("mux", P_double),
        ("kv_eta", P_double),
        ("kd2_form", c_int),
        ("rmass", P_double),
        ("nabs", c_int), ("abs_node", P_int), ("abs_C", P_double),
        ("time_scheme", c_int), ("dt", c_double), ("beta", c_double), ("gamma", c_double),
        ("nt", c_int),
        ("nsrc", c_int), ("src_node", P_int), ("src_dir", P_double), ("src_f0", P_double),
        ("src_t0", P_double), ("src_ampli", P_double), ("src_relamp", P_double),
        ("src_tdelay", P_double),
        ("nrec", c_int), ("rec_field", c_char), ("rec_isamp", c_int), ("rec_nsamp", c_int),
        ("rec_node", P_int), ("rec_elem", P_int), ("rec_interp", P_double),
        ("nflt", c_int), ("flt_node1", P_int), ("flt_node2", P_int), ("flt_n1", P_double),
        ("flt_B", P_double), ("flt_invM1", P_double), ("flt_invM2", P_double),
        ("flt_Z", P_double), ("flt_T0", P_double), ("flt_cohesion", P_double),
        ("flt_coefA2V", c_double), ("flt_coefA2D", c_double),
        ("flt_opening", c_int), ("flt_friction", c_int),
        ("swf_kind", c_int), ("swf_healing", c_int),
        ("swf_dc", P_double), ("swf_mus", P_double), ("swf_mud", P_double),
        ("swf_p", P_double), ("swf_alpha", P_double),
        ("rsf_kind", c_int),
        ("rsf_dc", P_double), ("rsf_mus", P_double), ("rsf_a", P_double), ("rsf_b", P_double),
        ("rsf_vstar", P_double), ("rsf_vc", P_double), ("rsf_theta", P_double),
        ("flt_V0", P_double),
        ("normal_kind", c_int), ("normal_T", c_double), ("normal_L", c_double),
        ("normal_V", c_double),
        ("flt_oit", c_int), ("flt_oitd", c_int), ("flt_oix1", c_int), ("flt_oixn", c_int),
        ("flt_oixd", c_int), ("flt_nsamp", c_int),
        ("precision", c_int),
        ("width", c_double),
        ("twf_kind", c_int),
        ("twf_mus", c_double), ("twf_mud", c_double), ("twf_mu0", c_double),
        ("twf_X", c_double), ("twf_Z", c_double), ("twf_V", c_double), ("twf_L", c_double),
        ("twf_T", c_double), ("twf_Dc", c_double),
        ("rho", P_double),
        ("adjoint", c_int),
        ("flt_potency", c_int),
        ("nstacey", c_int), ("stacey_node", P_int), ("stacey_k", P_int), ("stacey_edge", P_int),
        ("stacey_K", P_double),
        ("ndir", c_int), ("dir_node", P_int), ("dir_comp", P_int), ("dir_after_fault", P_int),
        ("alpha", c_double),
        ("nperio", c_int), ("perio_master", P_int), ("perio_slave", P_int),
        ("flt_nr_maxit", c_int), ("info_every", c_int),
        ("src_stf", P_Stf),
        ("wave_phase", c_int), ("wave_angle", c_double), ("wave_ref", c_double * 2),
        ("wave_cp", c_double), ("wave_cs", c_double), ("wave_mu", c_double),
        ("wave_lambda", c_double), ("wave_tdelay", c_double), ("wave_stf", P_Stf),
        ("abs_B", P_double), ("abs_n", P_double), ("abs_wave", P_int),
        ("nneu", c_int), ("neu_node", P_int), ("neu_comp", P_int), ("neu_B", P_double),
        ("neu_stf", P_int), ("nneu_stf", c_int), ("neu_stfs", P_Stf),
        ("xjaci", P_double), ("dvol", P_double),
    ]


class Domain(C.Structure):
    _fields_ = [("tag", c_int), ("ex", c_int * 2), ("ez", c_int * 2)]


class Material(C.Structure):
    _fields_ = [("tag", c_int), ("aniso", c_int),
                ("rho", c_double), ("cp", c_double), ("cs", c_double),
                ("c11", c_double), ("c13", c_double), ("c33", c_double), ("c55", c_double),
                ("c66", c_double),
                ("hetero", c_int), ("kv", c_int), ("kv_eta", c_double), ("kv_etaxdt", c_int)]


class BC(C.Structure):
    _fields_ = [("kind", c_int), ("tag", c_int * 2), ("stacey", c_int), ("dirichlet", c_int),
                ("no_wave", c_int), ("hstf", Stf), ("vstf", Stf)]


class Deck(C.Structure):
    _fields_ = [
        ("ngll", c_int), ("ndof", c_int), ("fmax", c_double),
        ("xlim", c_double * 2), ("zlim", c_double * 2), ("nelem", c_int * 2),
        ("ezflt", c_int), ("fztag", c_int), ("fznz", c_int),
        ("ndomains", c_int), ("domains", Domain * MAX_DOMAINS),
        ("nmats", c_int), ("mats", Material * MAX_MATS),
        ("h_rho", P_double), ("h_cp", P_double), ("h_cs", P_double),
        ("h_c11", P_double), ("h_c13", P_double), ("h_c33", P_double), ("h_c55", P_double),
        ("h_c66", P_double), ("h_kveta", P_double),
        ("nbcs", c_int), ("bcs", BC * MAX_BCS),
        ("flt_friction", c_int), ("swf_kind", c_int), ("swf_healing", c_int),
        ("rsf_kind", c_int), ("normal_kind", c_int),
        ("normal_T", c_double), ("normal_L", c_double), ("normal_V", c_double),
        ("flt_opening", c_int), ("flt_ot1", c_double), ("flt_otd", c_double),
        ("flt_oxi", c_int * 3),
        ("flt_value", c_double * FP_NPARAM), ("flt_array", P_double * FP_NPARAM),
        ("time_kind", c_int), ("dt", c_double), ("courant", c_double),
        ("total_time", c_double), ("nsteps", c_int), ("beta", c_double), ("gamma", c_double),
        ("hht_alpha", c_double), ("hht_rho", c_double),
        ("nsrc", c_int), ("src_coord", P_double), ("src_tdelay", P_double),
        ("src_ampli", P_double),
        ("ricker_f0", c_double), ("ricker_onset", c_double), ("ricker_ampli", c_double),
        ("force_angle", c_double),
        ("rec_number", c_int), ("rec_first", c_double * 2), ("rec_last", c_double * 2),
        ("rec_coord", P_double), ("rec_atnode", c_int), ("rec_isamp", c_int),
        ("rec_field", c_char),
        ("precision", c_int), ("kd2_form", c_int),
        ("width", c_double),
        ("twf_kind", c_int),
        ("twf_mus", c_double), ("twf_mud", c_double), ("twf_mu0", c_double),
        ("twf_X", c_double), ("twf_Z", c_double), ("twf_V", c_double), ("twf_L", c_double),
        ("twf_T", c_double), ("twf_Dc", c_double),
        ("flt_potency", c_int),
        ("src_mech", c_int), ("src_M", c_double * 4), ("src_dip", c_double),
        ("stf", Stf), ("wave_angle", c_double), ("wave_phase", c_int),
        ("mesh_method", c_int), ("zmin", c_double), ("nlayer", c_int),
        ("layer_nz", c_int * MAX_LAYERS), ("layer_tag", c_int * MAX_LAYERS),
        ("layer_ngnod", c_int * MAX_LAYERS), ("layer_top", P_double * MAX_LAYERS),
    ]


class TuneEntry(C.Structure):
    """sem2d_tune_entry: a launch shape of the march kernels and its time."""
    _fields_ = [("chunk_rows", c_int), ("warps_per_cta", c_int), ("ms_per_step", c_double)]


class LatticeArgs(C.Structure):
    """sem2d_lattice_args: caller-owned device arrays in the lattice layout."""
    _fields_ = [
        ("ngll", c_int), ("ndof", c_int), ("precision", c_int),
        ("nx", c_int), ("nz", c_int), ("LX", c_int), ("LZ", c_int), ("pitch", c_int),
        ("row0", C.c_void_p), ("hprime", P_double), ("wgll", P_double),
        ("d", C.c_void_p), ("v", C.c_void_p), ("rmass", C.c_void_p),
        ("per_rm", C.c_void_p), ("per_Ca", C.c_void_p), ("per_Cb", C.c_void_p),
        ("mat_iso", c_int), ("mat", C.c_void_p * 4),
        ("xix", C.c_void_p), ("etaz", C.c_void_p), ("dxdxi", C.c_void_p), ("dzdeta", C.c_void_p),
        ("nsrc", c_int), ("src_I", C.c_void_p), ("src_J", C.c_void_p), ("src_amp", C.c_void_p),
        ("nt", c_int), ("step0", c_int), ("dt", c_double), ("kd2_form", c_int),
        ("status", C.c_void_p),
    ]
