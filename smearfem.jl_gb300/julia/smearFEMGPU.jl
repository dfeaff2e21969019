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

export assemble_system, gaussian_quadrature, basis_function, solve_dirichlet, GPUMatrix

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
    opts = SolveOpts(precision == :mixed ? 1 : 0, precond == :block_jacobi ? 1 : 0, rtol, maxit, 32, 0.1, 0, 0)
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

end # module
