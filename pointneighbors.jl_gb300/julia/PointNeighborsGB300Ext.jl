# PointNeighborsGB300Ext -- the Julia side of libpn_gb300 (include/pn_gb300.h), written as a
# package extension of PointNeighbors.jl (v0.6.7) loaded together with CUDA.jl.
#
# A user keeps building searches with the reference's constructors; `GB300Search(nhs)`
# hands such a search to the library by the fields the reference stores
# (src/nhs_grid.jl:67-75, src/cell_lists/full_grid.jl:30-35, src/vector_of_vectors.jl:3-31):
#   nhs.search_radius, nhs.periodic_box, nhs.update_strategy,
#   nhs.cell_list.min_corner / max_corner      (already padded by 1001//1000 * search_radius)
#   size(nhs.cell_list.linear_indices)         (cells per dimension)
#   size(nhs.cell_list.cells.backend, 1)       (DynamicVectorOfVectors capacity)
# through pn_create_from_grid, which takes them as they are.  initialize!, update! and
# foreach_point_neighbor then dispatch to the library for CuArray coordinates and a pair
# function the library implements; any other closure keeps the reference's own
# KernelAbstractions path (there is no CPU fallback inside the library).
#
# Point indices are 0-based at the C boundary.  Coordinates are the reference's T[d, N]
# matrices, passed as they are.  The library is asynchronous on the given stream; like the
# reference, every call here ends with a synchronisation (pn_sync), which also turns the
# library's sticky error word into the reference's exceptions.
module PointNeighborsGB300Ext

using PointNeighbors
using PointNeighbors: GridNeighborhoodSearch, FullGridCellList, DynamicVectorOfVectors,
                      ParallelUpdate, ParallelIncrementalUpdate, SemiParallelUpdate,
                      SerialIncrementalUpdate, SerialUpdate
using CUDA

const lib = get(ENV, "PN_GB300_LIB", joinpath(@__DIR__, "..", "_build", "libpn_gb300.so"))

# --------------------------------------------------------------------- C structs
# pn_config: field order and alignment as in include/pn_gb300.h
struct PnConfig
    ndims::Int32
    dtype::Int32                      # 0 Float32, 1 Float64
    search_radius::Float64
    min_corner::NTuple{3, Float64}
    max_corner::NTuple{3, Float64}
    periodic::Int32
    update_strategy::Int32            # 0 rebuild, 1 incremental
    periodic_min::NTuple{3, Float64}
    periodic_max::NTuple{3, Float64}
    n_points::Int64
    max_points_per_cell::Int32
    flags::Int32                      # 1 = Float32 radius over Float64 coordinates
end

struct PnCountParams
    counts::CuPtr{Int32}
end

struct PnNBodyParams
    masses::CuPtr{Cvoid}
    G::Float64
    accel::CuPtr{Cvoid}
end

struct PnWCSPHParams
    mass::Float64; h::Float64; c0::Float64; rho0::Float64; gamma_exp::Float64
    alpha::Float64; eps_visc::Float64; r_min::Float64
    density::CuPtr{Cvoid}; pressure::CuPtr{Cvoid}; velocity::CuPtr{Cvoid}
    accel::CuPtr{Cvoid}; reuse_state::Int32; pad_::Int32
end

const PN_F_COUNT = Int32(0)
const PN_F_NBODY_ACCEL = Int32(2)
const PN_F_WCSPH_DENSITY = Int32(4)
const PN_F_WCSPH_FORCE = Int32(5)

status_string(code) = unsafe_string(ccall((:pn_status_string, lib), Cstring, (Int32,), code))

# Status codes to the reference's exceptions: ArgumentError for construction, the exact
# error() messages of full_grid.jl:205-212 and vector_of_vectors.jl:114-121, BoundsError for
# a query whose neighbouring cells lie outside the grid.
function check(code)
    code == 0 && return nothing
    code == 2 && throw(ArgumentError(status_string(code)))
    code == 9 && throw(BoundsError())
    code == 5 && throw(MethodError(foreach_point_neighbor, ()))
    error(status_string(code))
end

pad3(v) = ntuple(k -> k <= length(v) ? Float64(v[k]) : 0.0, 3)

strategy_code(::Union{ParallelUpdate, SerialUpdate}) = Int32(0)
strategy_code(::Union{ParallelIncrementalUpdate, SemiParallelUpdate,
                      SerialIncrementalUpdate}) = Int32(1)

# --------------------------------------------------------------------- the search
mutable struct GB300Search{NDIMS, T}
    handle::Ptr{Cvoid}
    search_radius::T
end

# A reference-constructed GridNeighborhoodSearch over a FullGridCellList with the
# DynamicVectorOfVectors backend (the GPU-capable configuration), by its stored state.
function GB300Search(nhs::GridNeighborhoodSearch{NDIMS, <:Any,
                                                 <:FullGridCellList{<:DynamicVectorOfVectors}};
                     n_points = 0) where {NDIMS}
    (; cell_list, search_radius, periodic_box, update_strategy) = nhs
    T = typeof(search_radius)
    C = eltype(cell_list.min_corner)
    mixed = T == Float32 && C == Float64   # docs/literate/src/tut_gpu_usage.jl:38-50
    grid = zeros(Int64, 3)
    grid[1:NDIMS] .= size(cell_list.linear_indices)
    cfg = PnConfig(NDIMS, C == Float64 ? 1 : 0, Float64(search_radius),
                   pad3(cell_list.min_corner), pad3(cell_list.max_corner),
                   isnothing(periodic_box) ? 0 : 1, strategy_code(update_strategy),
                   isnothing(periodic_box) ? (0.0, 0.0, 0.0) : pad3(periodic_box.min_corner),
                   isnothing(periodic_box) ? (0.0, 0.0, 0.0) : pad3(periodic_box.max_corner),
                   n_points, size(cell_list.cells.backend, 1), mixed ? 1 : 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pn_create_from_grid, lib), Cint,
                (Ref{PnConfig}, Ptr{Int64}, Ref{Ptr{Cvoid}}), cfg, grid, h))
    s = GB300Search{NDIMS, T}(h[], search_radius)
    finalizer(x -> ccall((:pn_destroy, lib), Cint, (Ptr{Cvoid},), x.handle), s)
    return s
end

stream() = CUDA.stream().handle
sync(s) = check(ccall((:pn_sync, lib), Cint, (Ptr{Cvoid},), s.handle))

function PointNeighbors.initialize!(s::GB300Search, x, y::CuMatrix;
                                    eachindex_y = axes(y, 2), kwargs...)
    whole = eachindex_y == axes(y, 2)
    idx = whole ? nothing : CuArray(Int32.(collect(eachindex_y)) .- Int32(1))
    check(ccall((:pn_initialize, lib), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, Int64, CuPtr{Int32}, Int64, Ptr{Cvoid}),
                s.handle, pointer(y), size(y, 2), whole ? CU_NULL : pointer(idx),
                whole ? 0 : length(idx), stream()))
    sync(s)
    return s
end

function PointNeighbors.update!(s::GB300Search, x, y::CuMatrix;
                                points_moving = (true, true), eachindex_y = axes(y, 2),
                                kwargs...)
    whole = eachindex_y == axes(y, 2)
    idx = whole ? nothing : CuArray(Int32.(collect(eachindex_y)) .- Int32(1))
    check(ccall((:pn_update, lib), Cint,
                (Ptr{Cvoid}, CuPtr{Cvoid}, Int64, CuPtr{Int32}, Int64, Int32, Ptr{Cvoid}),
                s.handle, pointer(y), size(y, 2), whole ? CU_NULL : pointer(idx),
                whole ? 0 : length(idx), Int32(points_moving[2]), stream()))
    sync(s)
    return s
end

PointNeighbors.requires_update(::GB300Search) = (false, true)

# --------------------------------------------------------------------- pair functions
# A pair function the library implements is a struct naming the functor and holding its
# output arrays; a closure is not one of them and is left to the reference.
struct CountNeighbors
    counts::CuVector{Int32}
end

struct NBodyAcceleration{T}
    masses::CuVector{T}
    G::T
    accel::CuMatrix{T}
end

struct WCSPHDensity{T}
    density::CuVector{T}; pressure::CuVector{T}; velocity::CuMatrix{T}
    mass::Float64; h::Float64; c0::Float64; rho0::Float64; gamma::Float64
end

struct WCSPHForce{T}
    density::CuVector{T}; pressure::CuVector{T}; velocity::CuMatrix{T}; accel::CuMatrix{T}
    mass::Float64; h::Float64; c0::Float64; rho0::Float64; gamma::Float64; alpha::Float64
    reuse_state::Bool
end

params(f::CountNeighbors) = (PN_F_COUNT, PnCountParams(pointer(f.counts)))
params(f::NBodyAcceleration) = (PN_F_NBODY_ACCEL,
                                PnNBodyParams(pointer(f.masses), Float64(f.G), pointer(f.accel)))
params(f::WCSPHDensity) = (PN_F_WCSPH_DENSITY,
                           PnWCSPHParams(f.mass, f.h, f.c0, f.rho0, f.gamma, 0.0, 0.01, 0.0,
                                         pointer(f.density), pointer(f.pressure),
                                         pointer(f.velocity), CU_NULL, 0, 0))
params(f::WCSPHForce) = (PN_F_WCSPH_FORCE,
                         PnWCSPHParams(f.mass, f.h, f.c0, f.rho0, f.gamma, f.alpha, 0.01,
                                       sqrt(eps(Float32)) * f.h, pointer(f.density),
                                       pointer(f.pressure), pointer(f.velocity),
                                       pointer(f.accel), f.reuse_state, 0))

const LibraryFunctor = Union{CountNeighbors, NBodyAcceleration, WCSPHDensity, WCSPHForce}

function PointNeighbors.foreach_point_neighbor(f::LibraryFunctor, x::CuMatrix, y::CuMatrix,
                                               s::GB300Search; points = axes(x, 2),
                                               kwargs...)
    functor, p = params(f)
    whole = points == axes(x, 2)
    pts = whole ? nothing : CuArray(Int32.(collect(points)) .- Int32(1))
    check(ccall((:pn_foreach_point_neighbor, lib), Cint,
                (Ptr{Cvoid}, Int32, CuPtr{Cvoid}, Int64, CuPtr{Cvoid}, Int64, CuPtr{Int32},
                 Int64, Ref{typeof(p)}, Ptr{Cvoid}),
                s.handle, functor, pointer(x), size(x, 2), pointer(y), size(y, 2),
                whole ? CU_NULL : pointer(pts), whole ? 0 : length(pts), p, stream()))
    sync(s)
    return nothing
end

end # module
