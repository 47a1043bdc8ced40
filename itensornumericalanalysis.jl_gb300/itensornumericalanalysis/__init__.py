"""GB300-native engine for quantics tensor network functions.

The public names follow ITensorNumericalAnalysis.jl (src/ITensorNumericalAnalysis.jl:20-66).
All tensor arithmetic runs in libtnfa (CUDA, sm_103a) behind the C ABI of
include/tnfa.h; this package holds the host-side graph / digit-map logic and
the constructors that write closed-form tensors.
"""
from . import _lib
from ._lib import Context, TnfaError, default_context, set_default_context
from .elementary_functions import (
    const_itensornetwork,
    const_itn,
    cos_itensornetwork,
    cos_itn,
    cosh_itensornetwork,
    cosh_itn,
    delta_kernel,
    delta_p,
    exp_itensornetwork,
    exp_itn,
    poly_itn,
    polynomial_itensornetwork,
    rand_itn,
    random_itensornetwork,
    sin_itensornetwork,
    sin_itn,
    sinh_itensornetwork,
    sinh_itn,
    tanh_itensornetwork,
    tanh_itn,
)
from .elementary_operators import (
    ITensorNetworkOperator,
    OpSum,
    backward_shift_op,
    backward_shift_opsum,
    first_derivative_operator,
    forward_shift_op,
    forward_shift_opsum,
    fourth_derivative_operator,
    identity_operator,
    laplacian_operator,
    map_to_zero_operator,
    map_to_zeros,
    multiply,
    operator_proj,
    opsum_to_operator,
    second_derivative_operator,
    stencil,
    third_derivative_operator,
    ttn,
)
from .graphs import (
    NamedGraph,
    named_binary_tree,
    named_comb_tree,
    named_grid,
    named_path_graph,
    uniform_tree,
)
from .indexmap import (
    AbstractIndexMap,
    ComplexIndexMap,
    ComplexIndsNetworkMap,
    IndsNetworkMap,
    RealIndexMap,
    RealIndsNetworkMap,
    SiteLeg,
    calculate_ind_values,
    calculate_p,
    complex_continuous_siteinds,
    complex_digit_siteinds,
    continuous_siteinds,
    default_dimension_vertices,
    digit_siteinds,
    dimension,
    dimension_inds,
    dimension_vertices,
    dimensions,
    grid_points,
    indexmap,
    indexmaptype,
    indsnetwork,
    merge_to_tree_image,
    real_continuous_siteinds,
    reduced_indsnetworkmap,
    tree_groups,
    base,
    digit,
    index_value_to_scalar,
    indsnetworkmap,
    vertex,
    vertex_digit,
    vertex_digits,
    vertex_dimension,
    vertex_dimensions,
    vertices_digits,
    vertices_dimensions,
)
from .grad import TTNEvaluate, evaluate_vjp
from .integration import integrate, partial_integrate
from .network import ITensorNetworkFunction, calculate_fx, evaluate, inner, itensornetwork
from .operate import operate, operate_batched, operate_exact, operate_vjp
from .solvers import dmrg, linsolve
from .tci import interpolate
from .truncation import truncate, truncate_batched

__version__ = "0.1.0"
