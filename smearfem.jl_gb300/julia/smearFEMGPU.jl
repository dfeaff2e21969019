"""
    smearFEMGPU

Drop-in GPU backend for the hot path of smearFEM.jl: `assemble_system` with
the reference's signature (src/fem.jl:135) and the Dirichlet solve of
examples/vector3D.jl:314-322, bound through `ccall` to libsmearfem_gpu.so
(include/smearfem_gpu.h).  `gaussian_quadrature` and `basis_function` are the
library's host-side helpers with the reference's expressions.

Set `ENV["SMEARFEM_GPU_LIB"]` to the path of libsmearfem_gpu.so before
`using smearFEMGPU` if it is not next to this file's `../lib/`.
"""
module smearFEMGPU

using SparseArrays

export assemble_system, gaussian_quadrature, basis_function, solve_dirichlet, GPUMatrix,
       apply_boundary_conditions!, solve_increments, meshgrid, inflate_sphere, write_vtk, write_scene,
       multigrid_info

const libsfem = get(ENV, "SMEARFEM_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libsmearfem_gpu.so"))

const SFEM_OK = Cint(0)
const SFEM_MEM_HOST = Cint(0)
const SFEM_Q1 = Cint(1)
const SFEM_Q2 = Cint(2)

struct SolveOpts
    precision::Cint
    precond::Cint
    rtol::Cdouble
    maxit::Cint
    check_every::Cint
    reliable_delta::Cdouble
    profile::Cint
    fp32_storage::Cint
end

# :jacobi, :block_jacobi, or :multigrid (mixed precision on meshgrid meshes; block Jacobi elsewhere)
_precond(p::Symbol) = p === :jacobi ? Cint(0) : p === :block_jacobi ? Cint(1) : p === :multigrid ? Cint(2) :
    throw(ArgumentError("precond must be :jacobi, :block_jacobi or :multigrid"))

mutable struct SolveStats
    status::Cint
    iterations::Cint
    reliable_updates::Cint
    relres::Cdouble
    ms_total::Cdouble
    ms_spmv::Cdouble
    spmv_launches::Cint
    kernel_launches::Cint
    n_free::Int64
    SolveStats() = new(0, 0, 0, 0.0, 0.0, 0.0, 0, 0, 0)
end

mutable struct Context
    h::Ptr{Cvoid}
end

const _ctx = Ref{Union{Nothing,Context}}(nothing)

function context()
    if _ctx[] === nothing
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:sfem_ctx_create, libsfem), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, h)
        st == SFEM_OK || error("smearFEMGPU: no usable GPU (status $st)")
        c = Context(h[])
        finalizer(x -> ccall((:sfem_ctx_destroy, libsfem), Cint, (Ptr{Cvoid},), x.h), c)
        _ctx[] = c
    end
    return _ctx[]::Context
end

function check(st, ctx::Context)
    if st != SFEM_OK
        msg = unsafe_string(ccall((:sfem_last_error, libsfem), Cstring, (Ptr{Cvoid},), ctx.h))
        st == 2 && throw(BoundsError(msg))               # bad IEN/ID index
        (st == 3 || st == 7) && throw(SingularException(0)) # inv of a singular matrix
        error("smearFEMGPU: $msg")
    end
end

"""GPU-resident stiffness matrix (keeps its mesh alive)."""
mutable struct GPUMatrix
    h::Ptr{Cvoid}
    n::Int64
    nnz::Int64
end

function _free(K::GPUMatrix)
    K.h != C_NULL && ccall((:sfem_matrix_destroy, libsfem), Cint, (Ptr{Cvoid},), K.h)
    K.h = C_NULL
end

function gaussian_quadrature(a, b, nGaussPoints=2)
    ξ = zeros(nGaussPoints); w = zeros(nGaussPoints)
    st = ccall((:sfem_gaussian_quadrature, libsfem), Cint,
               (Cdouble, Cdouble, Cint, Ptr{Cdouble}, Ptr{Cdouble}), a, b, nGaussPoints, ξ, w)
    st == SFEM_OK || error("nGaussPoints must be 2 or 3")
    return ξ, w
end

function basis_function(ξ, η=nothing, ζ=nothing, FunctionClass="Q1")
    ndim = ζ !== nothing ? 3 : (η !== nothing ? 2 : 1)
    fc = FunctionClass == "Q2" ? SFEM_Q2 : SFEM_Q1
    nen = fc == SFEM_Q2 ? 9 : 2^ndim
    N = zeros(nen); ΔN = zeros(nen, ndim)
    st = ccall((:sfem_basis_function, libsfem), Cint,
               (Cint, Cint, Cdouble, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Cdouble}),
               ndim, fc, ξ, something(η, 0.0), something(ζ, 0.0), N, ΔN)
    st == SFEM_OK || error("basis_function: $FunctionClass undefined in $(ndim)D")
    return N, (ndim == 1 ? reshape(ΔN, 1, 2) : ΔN)
end

"""
    assemble_system(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1, ID=nothing, Young=1, ν=0.3;
                    plane=:stress, handle=false)

Same arguments and result as smearFEM's `assemble_system` (src/fem.jl:135):
a `SparseMatrixCSC{Float64,Int64}`.  `handle=true` returns the `GPUMatrix`
instead, for `solve_dirichlet` without a host round trip.
"""
function assemble_system(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1, ID=nothing, Young=1, ν=0.3;
                         plane=:stress, handle=false)
    ctx = context()
    X = convert(Matrix{Float64}, NodeList)
    E = convert(Matrix{Int64}, IEN)
    I = ID === nothing ? C_NULL : convert(Matrix{Int64}, ID)
    Y = Float64.(vec(collect(Young)))
    V = Float64.(vec(collect(ν)))
    h = Ref{Ptr{Cvoid}}(C_NULL); n = Ref{Int64}(0); nnz = Ref{Int64}(0)
    fc = FunctionClass == "Q2" ? SFEM_Q2 : SFEM_Q1
    GC.@preserve X E I Y V begin
        st = ccall((:sfem_assemble_system, libsfem), Cint,
                   (Ptr{Cvoid}, Int64, Ptr{Cdouble}, Int64, Ptr{Int64}, Int64, Cint, Cint, Cint, Cint,
                    Ptr{Int64}, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64, Cint, Cint,
                    Ref{Ptr{Cvoid}}, Ref{Int64}, Ref{Int64}),
                   ctx.h, ne, X, size(X, 2), E, size(E, 1), size(E, 2), ndim, fc, nDof,
                   I, Y, length(Y), V, length(V), plane == :strain ? 1 : 0, SFEM_MEM_HOST, h, n, nnz)
    end
    check(st, ctx)
    K = GPUMatrix(h[], n[], nnz[])
    finalizer(_free, K)
    handle && return K
    return SparseMatrixCSC(K)
end

function SparseArrays.SparseMatrixCSC(K::GPUMatrix)
    ctx = context()
    colptr = Vector{Int64}(undef, K.n + 1)
    rowval = Vector{Int64}(undef, K.nnz)
    nzval = Vector{Float64}(undef, K.nnz)
    st = ccall((:sfem_matrix_export_csc, libsfem), Cint,
               (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Cdouble}, Cint),
               ctx.h, K.h, colptr, rowval, nzval, SFEM_MEM_HOST)
    check(st, ctx)
    return SparseMatrixCSC(K.n, K.n, colptr, rowval, nzval)
end

"""
    solve_dirichlet(K::GPUMatrix, fixed_dofs, fixed_vals, f=nothing; precision=:fp64, precond=:jacobi,
                    rtol=1e-10, maxit=100000)

`q = q_d + C*(K_free \\ C'*(f - K*q_d))`, the elimination of examples/vector3D.jl:314-322,
solved by preconditioned CG on the GPU.
"""
function solve_dirichlet(K::GPUMatrix, fixed_dofs, fixed_vals, f=nothing; precision=:fp64,
                         precond=:jacobi, rtol=1e-10, maxit=100000)
    ctx = context()
    fd = Int64.(collect(fixed_dofs)); fv = Float64.(collect(fixed_vals))
    fp = f === nothing ? C_NULL : Float64.(collect(f))
    u = Vector{Float64}(undef, K.n)
    opts = SolveOpts(precision == :mixed ? 1 : 0, _precond(precond), rtol, maxit, 32, 0.1, 0, 0)
    stats = SolveStats()
    GC.@preserve fd fv fp u begin
        st = ccall((:sfem_solve_dirichlet, libsfem), Cint,
                   (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                    Cint, Ref{SolveOpts}, Ref{SolveStats}),
                   ctx.h, K.h, fd, length(fd), fv, fp, u, SFEM_MEM_HOST, opts, stats)
    end
    check(st, ctx)
    return u
end

"""
    apply_boundary_conditions!(K::GPUMatrix, NodeList, IEN_top, IEN_btm, β)

`K_bar = K + β*b` in place on the GPU, where `b` is the surface penalty of
`apply_boundary_conditions` (examples/vector3D.jl:175-264, 306-308) computed on
the face coordinates `NodeList` (the driver passes the inflated cylinder).
"""
function apply_boundary_conditions!(K::GPUMatrix, NodeList, IEN_top, IEN_btm, β)
    ctx = context()
    X = convert(Matrix{Float64}, NodeList)
    F = vcat(convert(Matrix{Int64}, IEN_btm), convert(Matrix{Int64}, IEN_top))   # the reference's COO order
    GC.@preserve X F begin
        st = ccall((:sfem_penalty_add, libsfem), Cint,
                   (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Int64}, Int64, Cint, Cdouble, Cint),
                   ctx.h, K.h, X, F, size(F, 1), size(F, 2), β, SFEM_MEM_HOST)
    end
    check(st, ctx)
    return K
end

"""
    solve_increments(K::GPUMatrix, fixed_dofs, fixed_vals::Matrix; warm_start=true, precision=:fp64,
                     precond=:jacobi, rtol=1e-10, maxit=100000)

The load-increment loop of examples/vector3D.jl:310-338: column `s` of
`fixed_vals` (nfix × nsteps) holds step s's prescribed values; returns the
n × nsteps displacements.  With `warm_start` each step starts from the best
affine combination of up to three earlier solutions.
"""
function solve_increments(K::GPUMatrix, fixed_dofs, fixed_vals::AbstractMatrix; warm_start=true,
                          precision=:fp64, precond=:jacobi, rtol=1e-10, maxit=100000)
    ctx = context()
    fd = Int64.(collect(fixed_dofs)); fv = convert(Matrix{Float64}, fixed_vals)
    nsteps = size(fv, 2)
    U = Matrix{Float64}(undef, K.n, nsteps)
    opts = SolveOpts(precision == :mixed ? 1 : 0, _precond(precond), rtol, maxit, 32, 0.1, 0, 0)
    GC.@preserve fd fv U begin
        st = ccall((:sfem_solve_increments, libsfem), Cint,
                   (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Ptr{Cdouble},
                    Cint, Ref{SolveOpts}, Cint, Ptr{Cvoid}),
                   ctx.h, K.h, fd, length(fd), fv, nsteps, C_NULL, U, SFEM_MEM_HOST, opts, warm_start ? 1 : 0,
                   C_NULL)
    end
    check(st, ctx)
    return U
end

"""
    multigrid_info(nNodes, IEN, ndim; nDof=ndim, FunctionClass="Q1")

Whether `precond=:multigrid` gives this mesh a hierarchy (host only, no GPU):
`(ne, levels, bytes)` with `ne` the elements per direction of a meshgrid mesh
(0 for any other mesh) and the hierarchy's levels and device bytes.
"""
function multigrid_info(nNodes, IEN::AbstractMatrix, ndim; nDof=ndim, FunctionClass="Q1")
    I = Matrix{Int64}(IEN)
    ne = Ref{Cint}(0); lv = Ref{Cint}(0); nb = Ref{Int64}(0)
    fc = FunctionClass == "Q2" ? SFEM_Q2 : SFEM_Q1
    st = GC.@preserve I ccall((:sfem_multigrid_info, libsfem), Cint,
                              (Cint, Cint, Cint, Int64, Ptr{Int64}, Int64, Ref{Cint}, Ref{Cint}, Ref{Int64}),
                              ndim, fc, nDof, nNodes, I, size(I, 1), ne, lv, nb)
    st == SFEM_OK || throw(ErrorException("sfem_multigrid_info: status $st"))
    return (ne = Int(ne[]), levels = Int(lv[]), bytes = nb[])
end

"""
    meshgrid(x0, x1, y0, y1, z0, z1, ne, ndim)

The driver's mesh generator (examples/vector3D.jl:10-130) run on the GPU:
`NodeList, IEN, ID, IEN_top, IEN_btm` in the reference's shapes.
"""
function meshgrid(x0, x1, y0, y1, z0, z1, ne, ndim)
    ctx = context()
    nN = (ne + 1)^ndim; nEl = ne^ndim; nF = ne^(ndim - 1); nenF = 2^(ndim - 1)
    NodeList = Matrix{Float64}(undef, ndim, nN)
    IEN = Matrix{Int64}(undef, nEl, 2^ndim); ID = Matrix{Int64}(undef, nN, ndim)
    IEN_top = Matrix{Int64}(undef, nF, nenF); IEN_btm = Matrix{Int64}(undef, nF, nenF)
    st = ccall((:sfem_meshgrid, libsfem), Cint,
               (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Int64, Cint,
                Ptr{Cdouble}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Cint),
               ctx.h, x0, x1, y0, y1, z0, z1, ne, ndim, NodeList, IEN, ID, IEN_top, IEN_btm, SFEM_MEM_HOST)
    check(st, ctx)
    return NodeList, IEN, ID, IEN_top, IEN_btm
end

"""
    inflate_sphere(NodeList, x0, x1, y0, y1)

src/PostProcess.jl:30-44 on the GPU; like the reference it changes `NodeList`
in place and returns it.
"""
function inflate_sphere(NodeList::Matrix{Float64}, x0, x1, y0, y1)
    ctx = context()
    st = ccall((:sfem_inflate_sphere, libsfem), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Int64, Cdouble, Cdouble, Cdouble, Cdouble, Cint),
               ctx.h, NodeList, size(NodeList, 1), size(NodeList, 2), x0, x1, y0, y1, SFEM_MEM_HOST)
    check(st, ctx)
    return NodeList
end

"""
    write_vtk(fileName, fieldName, NodeList, IEN, ne, ndim, q)

src/PostProcess.jl:258-279: `fileName.vtu` with the cells `IEN[1:ne^ndim, :]` and
the point field `q` (one value per node, or a components × nodes matrix).
"""
function write_vtk(fileName, fieldName, NodeList, IEN, ne, ndim, q)
    X = convert(Matrix{Float64}, NodeList); E = convert(Matrix{Int64}, IEN[1:ne^ndim, :])
    Q = convert(Array{Float64}, q)
    ncomp = ndims(Q) == 1 ? 1 : size(Q, 1)
    st = ccall((:sfem_vtk_write, libsfem), Cint,
               (Ptr{Cvoid}, Cstring, Ptr{Cdouble}, Cint, Int64, Ptr{Int64}, Int64, Cint, Cstring,
                Ptr{Cdouble}, Cint, Cint),
               C_NULL, string(fileName, ".vtu"), X, size(X, 1), size(X, 2), E, size(E, 1), size(E, 2),
               string(fieldName), Q, ncomp, SFEM_MEM_HOST)
    st == SFEM_OK || error("smearFEMGPU: writing $fileName.vtu failed (status $st)")
    return nothing
end

"""
    write_scene(fileName, NodeList, IEN, ne, ndim, fields)

src/PostProcess.jl:281-304: `fileName` * "timestep_i.vtu" per field (point data
"u") and `fileName` * "displacement.pvd" listing them at times 0, 1, ...
"""
function write_scene(fileName, NodeList, IEN, ne, ndim, fields)
    X = convert(Matrix{Float64}, NodeList); E = convert(Matrix{Int64}, IEN[1:ne^ndim, :])
    F = reduce(vcat, [vec(convert(Array{Float64}, f)) for f in fields])
    ncomp = ndims(fields[1]) == 1 ? 1 : size(fields[1], 1)
    st = ccall((:sfem_vtk_write_scene, libsfem), Cint,
               (Ptr{Cvoid}, Cstring, Ptr{Cdouble}, Cint, Int64, Ptr{Int64}, Int64, Cint, Ptr{Cdouble}, Cint,
                Int64, Cint),
               C_NULL, string(fileName), X, size(X, 1), size(X, 2), E, size(E, 1), size(E, 2), F, ncomp,
               length(fields), SFEM_MEM_HOST)
    st == SFEM_OK || error("smearFEMGPU: writing the scene $fileName failed (status $st)")
    return nothing
end

end # module
