#
# SEMB200.jl — Julia binding of libsem_b200.so: new methods of SpectralElements.jl's
# operator/solve functions for CuArray fields, calling the C ABI of
# include/sem_b200.h through ccall.  Host Arrays keep using the package's own
# CPU methods; CuArrays never take a CPU or CUDA.jl-broadcast path.
#
# Usage (after `using SpectralElements, CUDA`):
#   include("SEMB200.jl"); using .SEMB200
#   u  = CuArray(msh.x)                  # any local field of the mesh
#   Au = lapl(u, msh)                    # -> sem_lapl
#   op = SEMB200.HelmholtzOp(msh, ν, k, ['D','D','D','D'])
#   x  = pcg(b, op; opM=SEMB200.Jacobi(op), mult=msh.mult, tol=1e-8)
#
module SEMB200

using CUDA
import ChainRulesCore
import SpectralElements: ABu, lapl, mass, hlmz, gatherScatter, mask, pcg, pcg!, Mesh, generateMask,
                         linsolve
using LinearAlgebra: I

const libsem = get(ENV, "SEM_B200_LIB", joinpath(@__DIR__, "..", "lib", "libsem_b200.so"))

const SEM_OK = Cint(0)
const SEM_ERR_NOT_CONVERGED = Cint(2)
const SEM_GS = Cuint(1)
const SEM_MASK = Cuint(2)
const SEM_F64 = Cint(0)
const SEM_F64_DF = Cint(1)
const SEM_MIXED = Cint(3)
const SEM_MIXED_RR = Cint(4)
const SEM_PATH_AUTO = Cint(0)
const SEM_PATH_CHUNKED = Cint(1)
const SEM_PATH_SMALL = Cint(2)

struct MeshDesc
    nr::Cint; ns::Cint; Ex::Cint; Ey::Cint
    periodic_x::Cint; periodic_y::Cint
    Dr::Ptr{Cdouble}; Ds::Ptr{Cdouble}; wr::Ptr{Cdouble}; ws::Ptr{Cdouble}
    x::Ptr{Cdouble}; y::Ptr{Cdouble}
    G11::Ptr{Cdouble}; G12::Ptr{Cdouble}; G22::Ptr{Cdouble}; B::Ptr{Cdouble}
    bc::Ptr{UInt8}
end

struct PcgOpts
    nu::Cdouble; nu_field::CuPtr{Cdouble}; k::Cdouble
    precond::Cint; precision::Cint; tol::Cdouble; maxiter::Cint
    inner_tol::Cdouble; max_outer::Cint; check_every::Cint; mult_ones::Cint; path::Cint
end

# immutable (isbits), so that a Vector{SolveInfo} is a C array of records;
# single results are read through Ref{SolveInfo}
struct SolveInfo
    iters::Cint; outer::Cint; res_inf::Cdouble; res0_inf::Cdouble; converged::Cint
end
SolveInfo() = SolveInfo(0, 0, 0.0, 0.0, 0)

lasterr() = unsafe_string(ccall((:sem_last_error, libsem), Cstring, ()))
check(st) = st == SEM_OK || error("libsem_b200 status $st: $(lasterr())")
stream() = CUDA.stream().handle

# Mesh -> device handle cache: the Julia Mesh is immutable, so the handle is
# built once from its host arrays (geometry uploaded verbatim).
const HANDLES = IdDict{Any,Ptr{Cvoid}}()

function handle(msh::Mesh)
    get!(HANDLES, msh) do
        d = Ref(MeshDesc(msh.nr, msh.ns, msh.Ex, msh.Ey, msh.ifperiodic[1], msh.ifperiodic[2],
                         pointer(msh.Dr), pointer(msh.Ds), pointer(msh.wr), pointer(msh.ws),
                         pointer(msh.x), pointer(msh.y), pointer(msh.G11), pointer(msh.G12),
                         pointer(msh.G22), pointer(msh.B), Ptr{UInt8}(C_NULL)))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve msh check(ccall((:sem_mesh_create, libsem), Cint,
                                     (Ref{MeshDesc}, Ref{Ptr{Cvoid}}), d, h))
        finalizer(m -> ccall((:sem_mesh_destroy, libsem), Cint, (Ptr{Cvoid},), h[]), msh)
        h[]
    end
end

set_bc!(msh::Mesh, bc::Vector{Char}) =
    check(ccall((:sem_mesh_set_bc, libsem), Cint, (Ptr{Cvoid}, Cstring), handle(msh), String(bc)))

# ---- kernel-variant autotuner (no counterpart in the reference): times every
# variant of the fused element operator on this mesh and keeps the fastest
const SEM_VARIANTS = 6
function autotune!(msh::Mesh; precision=SEM_F64_DF)
    ms = zeros(Cdouble, SEM_VARIANTS)
    chosen = Ref{Cint}(0)
    check(ccall((:sem_mesh_autotune, libsem), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ref{Cint}),
                handle(msh), precision, ms, chosen))
    return (chosen=Int(chosen[]), ms=ms)
end

# ---- ABu(As,Br,u) (src/ABu.jl:9-37); [] = identity
function ABu(As::AbstractArray, Br::AbstractArray, u::CuArray{Float64,2})
    m, n = size(u)
    A = length(As) == 0 ? nothing : Matrix{Float64}(As)
    B = length(Br) == 0 ? nothing : Matrix{Float64}(Br)
    mo = B === nothing ? m : div(m * size(B, 1), size(B, 2))
    no = A === nothing ? n : div(n, size(A, 2)) * size(A, 1)
    v = CuArray{Float64}(undef, mo, no)
    GC.@preserve A B check(ccall((:sem_abu, libsem), Cint,
        (Ptr{Cdouble}, Cint, Cint, Ptr{Cdouble}, Cint, Cint, CuPtr{Cdouble}, Cint, Cint,
         CuPtr{Cdouble}, Ptr{Cvoid}),
        A === nothing ? C_NULL : pointer(A), A === nothing ? 0 : size(A, 1), A === nothing ? 0 : size(A, 2),
        B === nothing ? C_NULL : pointer(B), B === nothing ? 0 : size(B, 1), B === nothing ? 0 : size(B, 2),
        pointer(u), m, n, pointer(v), stream()))
    return v
end

# ---- lapl(u,msh), lapl(u,ν,msh), mass, hlmz, gatherScatter, mask
function lapl(u::CuArray{Float64,2}, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_lapl, libsem), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), pointer(u), pointer(out), 0, stream()))
    return out
end

function lapl(u::CuArray{Float64,2}, ν::CuArray{Float64,2}, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_lapl_nu, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), pointer(ν), pointer(u), pointer(out), 0, stream()))
    return out
end

function mass(u::CuArray{Float64,2}, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_mass, libsem), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), pointer(u), pointer(out), 0, stream()))
    return out
end

function hlmz(u::CuArray{Float64,2}, ν::Number, k::Number, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_hlmz, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), CU_NULL, ν, k, pointer(u), pointer(out), 0, stream()))
    return out
end

function hlmz(u::CuArray{Float64,2}, ν::CuArray{Float64,2}, k::Number, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_hlmz, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), pointer(ν), 1.0, k, pointer(u), pointer(out), 0, stream()))
    return out
end

function gatherScatter(u::CuArray{Float64,2}, msh::Mesh)
    out = similar(u)
    check(ccall((:sem_gather_scatter, libsem), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cvoid}),
                handle(msh), pointer(u), pointer(out), stream()))
    return out
end

# ---- functional forms on explicit operands (no Mesh): the calls of
# examples/p2d_explicit.jl:183-190 and examples/semPS.jl:157-175.
# QQtx/QQty are the reference's host gather-scatter matrices (Q Q' of semq);
# their numbering (points per element, elements, periodicity) is read from
# their couplings, and the sums run on the device without the matrices.
# An empty QQtx/QQty ([]) leaves the field unassembled, an empty M unmasked,
# empty Jr/Js select the plain (not dealiased) quadrature, as in the reference.
function qq_structure(QQ::AbstractMatrix)
    NL = size(QQ, 1)
    size(QQ, 2) == NL || throw(ArgumentError("QQ must be square"))
    periodic = NL > 1 && QQ[1, NL] != 0
    n = NL
    for i in 2:NL-1                      # n >= 2: first interface between lines n and n+1
        if QQ[i, i+1] != 0
            n = i
            break
        end
    end
    NL % n == 0 || throw(ArgumentError("QQ is not the gather-scatter matrix of a semq numbering"))
    return n, div(NL, n), periodic
end

devarray(A::CuArray{Float64}) = A
devarray(A::AbstractArray) = CuArray{Float64}(Float64.(A))

# gatherScatter(u,QQtx,QQty) (src/gatherScatter.jl:8-16) -> sem_gather_scatter_grid
function gatherScatter(u::CuArray{Float64,2}, QQtx::AbstractMatrix, QQty::AbstractMatrix)
    nr, Ex, px = qq_structure(QQtx)
    ns, Ey, py = qq_structure(QQty)
    size(u) == (nr * Ex, ns * Ey) || throw(DimensionMismatch("u does not match QQtx/QQty"))
    out = similar(u)
    check(ccall((:sem_gather_scatter_grid, libsem), Cint,
                (Cint, Cint, Cint, Cint, Cint, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cvoid}),
                nr, ns, Ex, Ey, px, py, pointer(u), pointer(out), stream()))
    return out
end

function assemble_mask(v::CuArray{Float64,2}, M, QQtx, QQty)
    w = (length(QQtx) == 0 && length(QQty) == 0) ? v : gatherScatter(v, QQtx, QQty)
    return length(M) == 0 ? w : mask(w, devarray(M))
end

# functional lapl(u,M,Jr,Js,QQtx,QQty,Dr,Ds,G11,G12,G22,mult) (src/lapl.jl:54-68):
# plain quadrature -> sem_lapl_geom (the fused element operator), dealiased ->
# sem_laplace_dealiased; then QQ' (sem_gather_scatter_grid) and the mask
function lapl(u::CuArray{Float64,2}, M, Jr, Js, QQtx, QQty, Dr::AbstractMatrix, Ds::AbstractMatrix,
              G11::CuArray{Float64,2}, G12::CuArray{Float64,2}, G22::CuArray{Float64,2}, mult;
              precision=SEM_F64_DF)
    nr, ns = size(Dr, 1), size(Ds, 1)
    Ex, Ey = div(size(u, 1), nr), div(size(u, 2), ns)
    Drm, Dsm = Matrix{Float64}(Dr), Matrix{Float64}(Ds)
    out = similar(u)
    if length(Jr) == 0 && length(Js) == 0
        px = length(QQtx) > 0 && qq_structure(QQtx)[3]
        py = length(QQty) > 0 && qq_structure(QQty)[3]
        flags = length(QQtx) > 0 ? SEM_GS : Cuint(0)
        GC.@preserve Drm Dsm check(ccall((:sem_lapl_geom, libsem), Cint,
            (Cint, Cint, Cint, Cint, Cint, Cint, Cstring, Ptr{Cdouble}, Ptr{Cdouble}, CuPtr{Cdouble},
             CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Cint, Ptr{Cvoid}),
            nr, ns, Ex, Ey, px, py, C_NULL, Drm, Dsm, pointer(G11), pointer(G12), pointer(G22),
            pointer(u), pointer(out), flags, precision, stream()))
        return length(M) == 0 ? out : mask(out, devarray(M))
    end
    Jrm = length(Jr) == 0 ? Matrix{Float64}(I, nr, nr) : Matrix{Float64}(Jr)
    Jsm = length(Js) == 0 ? Matrix{Float64}(I, ns, ns) : Matrix{Float64}(Js)
    GC.@preserve Drm Dsm Jrm Jsm check(ccall((:sem_laplace_dealiased, libsem), Cint,
        (Cint, Cint, Cint, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
         CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cvoid}),
        nr, size(Jrm, 1), size(Jsm, 1), Ex, Ey, Jrm, Jsm, Drm, Dsm, pointer(G11), pointer(G12),
        pointer(G22), pointer(u), pointer(out), stream()))
    return assemble_mask(out, M, QQtx, QQty)
end

# functional mass(u,M,B,Jr,Js,QQtx,QQty,mult) (src/mass.jl:32-50):
# J'(B .* (J u)) (sem_mass_dealiased, or B .* u through sem_mask), QQ', mask
function mass(u::CuArray{Float64,2}, M, B, Jr, Js, QQtx, QQty, mult)
    out = similar(u)
    if length(Jr) == 0 && length(Js) == 0
        length(B) == 0 ? copyto!(out, u) : (out = mask(u, devarray(B)))
        return assemble_mask(out, M, QQtx, QQty)
    end
    n = length(Jr) == 0 ? size(Js, 2) : size(Jr, 2)
    Ex, Ey = div(size(u, 1), n), div(size(u, 2), n)
    Jrm = length(Jr) == 0 ? Matrix{Float64}(I, n, n) : Matrix{Float64}(Jr)
    Jsm = length(Js) == 0 ? Matrix{Float64}(I, n, n) : Matrix{Float64}(Js)
    Bd = length(B) == 0 ? nothing : devarray(B)
    GC.@preserve Jrm Jsm check(ccall((:sem_mass_dealiased, libsem), Cint,
        (Cint, Cint, Cint, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble},
         CuPtr{Cdouble}, Ptr{Cvoid}),
        n, size(Jrm, 1), size(Jsm, 1), Ex, Ey, Jrm, Jsm, Bd === nothing ? CU_NULL : pointer(Bd),
        pointer(u), pointer(out), stream()))
    return assemble_mask(out, M, QQtx, QQty)
end

# Pullbacks of the functional forms in u, with the reference's convention:
# the cotangent reaching the unassembled operator output is scaled by mult
# (the Zygote.hook(d -> d .* mult, .) of src/lapl.jl:62 and src/mass.jl:45),
# and laplace / J'BJ are symmetric, so the same device calls apply the
# transpose.  Cotangents of the geometry and operator matrices are not
# implemented here (the reference's own AD serves them on host arrays).
function ChainRulesCore.rrule(::typeof(lapl), u::CuArray{Float64,2}, M, Jr, Js, QQtx, QQty, Dr, Ds,
                              G11, G12, G22, mult; kw...)
    y = lapl(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22, mult; kw...)
    function lapl_pullback(ȳ)
        d = assemble_mask(CuArray{Float64,2}(ChainRulesCore.unthunk(ȳ)), M, QQtx, QQty)
        d = mask(d, devarray(mult))
        ū = lapl(d, [], Jr, Js, [], [], Dr, Ds, G11, G12, G22, mult; kw...)
        nt = ChainRulesCore.@not_implemented("geometry and operator cotangents of the device lapl")
        return (ChainRulesCore.NoTangent(), ū, ChainRulesCore.NoTangent(), nt, nt,
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), nt, nt, nt, nt, nt,
                ChainRulesCore.NoTangent())
    end
    return y, lapl_pullback
end

function ChainRulesCore.rrule(::typeof(mass), u::CuArray{Float64,2}, M, B, Jr, Js, QQtx, QQty, mult)
    y = mass(u, M, B, Jr, Js, QQtx, QQty, mult)
    function mass_pullback(ȳ)
        d = assemble_mask(CuArray{Float64,2}(ChainRulesCore.unthunk(ȳ)), M, QQtx, QQty)
        d = mask(d, devarray(mult))
        ū = mass(d, [], B, Jr, Js, [], [], mult)
        nt = ChainRulesCore.@not_implemented("B and interpolation cotangents of the device mass")
        return (ChainRulesCore.NoTangent(), ū, ChainRulesCore.NoTangent(), nt, nt, nt,
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return y, mass_pullback
end

function mask(u::CuArray{Float64,2}, M::CuArray{Float64,2})
    out = similar(u)
    check(ccall((:sem_mask, libsem), Cint, (CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Int64, Ptr{Cvoid}),
                pointer(M), pointer(u), pointer(out), length(u), stream()))
    return out
end

# ---- fused operator objects accepted by pcg (callable, so opA * u works
# through Base.:*(op::Function, x) of src/SpectralElements.jl:21)
struct HelmholtzOp <: Function
    msh::Mesh
    ν::Float64
    k::Float64
    bc::Vector{Char}
end
function (op::HelmholtzOp)(u::CuArray{Float64,2})
    set_bc!(op.msh, op.bc)
    out = similar(u)
    check(ccall((:sem_hlmz, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(op.msh), CU_NULL, op.ν, op.k, pointer(u), pointer(out), SEM_GS | SEM_MASK, stream()))
    return out
end

# opLHS on HOST arrays (the reference's own Array fields): the field streams to
# the GPU and back in slabs with the copies overlapped (sem_hlmz_host). Pin the
# arrays once (CUDA.Mem.pin) for the overlap; unpinned arrays work, with
# serialised copies.
function (op::HelmholtzOp)(out::Array{Float64,2}, u::Array{Float64,2}; slabs::Integer=0)
    set_bc!(op.msh, op.bc)
    check(ccall((:sem_hlmz_host, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Cdouble}, Cuint, Cint, Ptr{Cvoid}),
                handle(op.msh), CU_NULL, op.ν, op.k, u, out, SEM_GS | SEM_MASK, slabs, stream()))
    CUDA.synchronize()
    return out
end

struct Jacobi <: Function
    op::HelmholtzOp
end

# ---- pcg(b,opA;opM,mult,ifv,tol,maxiter) (src/pcg.jl:16-60) on the device
function pcg(b::CuArray{Float64,2}, opA::HelmholtzOp; opM=x -> x, mult=nothing, ifv=false,
             tol=1e-8, maxiter=length(b), precision=SEM_F64_DF)
    opM isa Jacobi || opM === identity || opM isa Function && !(opM isa HelmholtzOp) ||
        throw(ArgumentError("opM must be x->x or SEMB200.Jacobi(opA)"))
    set_bc!(opA.msh, opA.bc)
    x = similar(b)
    o = Ref(PcgOpts(opA.ν, CU_NULL, opA.k, opM isa Jacobi ? 1 : 0, precision, tol, maxiter,
                    1e-4, 6, 0, mult === nothing ? 1 : 0, 0))
    info = Ref(SolveInfo())
    st = ccall((:sem_pcg, libsem), Cint,
               (Ptr{Cvoid}, Ref{PcgOpts}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{SolveInfo}, Ptr{Cvoid}),
               handle(opA.msh), o, pointer(b), pointer(x), info, stream())
    if st == SEM_ERR_NOT_CONVERGED
        println("warning: res:", info[].res_inf)
        return x
    end
    check(st)
    ifv && println("PCG iter: ", info[].iters, ", res: ", info[].res_inf)
    return x
end

pcg(b::CuArray, opA::Function; kw...) =
    throw(ArgumentError("pcg on CuArrays takes a SEMB200 operator object; closures are not run on the host"))

function pcg!(x::CuArray{Float64,2}, b::CuArray{Float64,2}, opA::HelmholtzOp; kw...)
    x .= pcg(b, opA; kw...)
    return
end

# ---- batched solves: many independent Diffusion-type systems (different
# element counts, orders, ν and k) in one persistent launch per order
mutable struct BatchSolver
    ptr::Ptr{Cvoid}
    meshes::Vector{Mesh}
end
function BatchSolver(meshes::Vector{<:Mesh}, ν::Vector{Float64}, k::Vector{Float64},
                     bc::Vector{Char}; jacobi::Bool=true)
    hs = Ptr{Cvoid}[handle(m) for m in meshes]
    foreach(m -> set_bc!(m, bc), meshes)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sem_batch_create, libsem), Cint,
                (Ptr{Ptr{Cvoid}}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Cint, Ref{Ptr{Cvoid}}),
                hs, ν, k, length(meshes), jacobi ? 1 : 0, out))
    b = BatchSolver(out[], collect(meshes))
    finalizer(x -> ccall((:sem_batch_destroy, libsem), Cint, (Ptr{Cvoid},), x.ptr), b)
    return b
end
function solve(bs::BatchSolver, rhs::Vector{<:CuArray{Float64,2}}, tol::Vector{Float64};
               precision=SEM_F64_DF, inner_tol=1e-4, max_outer=6)
    xs = [similar(r) for r in rhs]
    bp = CuPtr{Cdouble}[pointer(r) for r in rhs]
    xp = CuPtr{Cdouble}[pointer(x) for x in xs]
    info = fill(SolveInfo(), length(rhs))
    st = ccall((:sem_batch_pcg, libsem), Cint,
               (Ptr{Cvoid}, Ptr{CuPtr{Cdouble}}, Ptr{CuPtr{Cdouble}}, Ptr{Cdouble}, Ptr{Cint}, Cint,
                Cdouble, Cint, Ptr{SolveInfo}, Ptr{Cvoid}),
               bs.ptr, bp, xp, tol, C_NULL, precision, inner_tol, max_outer, info, stream())
    st == SEM_ERR_NOT_CONVERGED && println("warning: some batched solves reached maxiter")
    st == SEM_ERR_NOT_CONVERGED || check(st)
    return xs, info
end

# ---- device time loop: nsteps of evolve! (src/diffusion.jl:81-106) in one
# sem_bdf_run call.  u and the histories uh are CuArrays of the mesh; time is
# the TimeStepper's time vector (updated in place); forcing and boundary are
# vectors of (field, t -> coefficient) pairs, the separable forms of the
# reference's setForcing!/setBC! closures.  The solve is the reference's
# Diffusion solve: identity preconditioner, mult = msh.mult, tol absolute.
struct BdfDesc
    order::Cint; nu::Cdouble; dt::Cdouble; nsteps::Cint
    solve::PcgOpts
    nf::Cint; F::Ptr{CuPtr{Cdouble}}; fcoef::Ptr{Cdouble}
    nb::Cint; UB::Ptr{CuPtr{Cdouble}}; bcoef::Ptr{Cdouble}
end
function bdf_run!(u::CuArray{Float64,2}, uh::Vector{<:CuArray{Float64,2}}, time::Vector{Float64},
                  msh::Mesh, bc::Vector{Char}, ν::Float64, dt::Float64, nsteps::Int;
                  forcing=Tuple{CuArray{Float64,2},Function}[],
                  boundary=Tuple{CuArray{Float64,2},Function}[],
                  tol=1e-8, precision=SEM_F64_DF, jacobi::Bool=false)
    set_bc!(msh, bc)
    k = length(uh)
    ts = Float64[]
    t = time[1]
    for _ in 1:nsteps
        t += dt
        push!(ts, t)
    end
    fc = Float64[fn(tt) for tt in ts for (_, fn) in forcing]
    bcf = Float64[fn(tt) for tt in ts for (_, fn) in boundary]
    F = CuPtr{Cdouble}[pointer(f) for (f, _) in forcing]
    UB = CuPtr{Cdouble}[pointer(g) for (g, _) in boundary]
    uhp = CuPtr{Cdouble}[pointer(v) for v in uh]
    info = fill(SolveInfo(), nsteps)
    GC.@preserve fc bcf F UB begin
        d = Ref(BdfDesc(k, ν, dt, nsteps,
                        PcgOpts(ν, CU_NULL, 0.0, jacobi ? 1 : 0, precision, tol, 0, 0.0, 0, 0, 0, 0),
                        length(forcing), pointer(F), pointer(fc),
                        length(boundary), pointer(UB), pointer(bcf)))
        st = ccall((:sem_bdf_run, libsem), Cint,
                   (Ptr{Cvoid}, Ref{BdfDesc}, Ptr{Cdouble}, CuPtr{Cdouble}, Ptr{CuPtr{Cdouble}},
                    Ptr{SolveInfo}, Ptr{Cvoid}),
                   handle(msh), d, time, pointer(u), uhp, info, stream())
    end
    st == SEM_ERR_NOT_CONVERGED && println("warning: some steps reached maxiter")
    st == SEM_ERR_NOT_CONVERGED || check(st)
    return info
end

# ---- differentiable solve of -div(ν grad u) + k u = f with ν folded into G
# (examples/semPS.jl:163-165), the pattern of linsolve + @adjoint in
# src/adjoint.jl:5-24 as ChainRulesCore rrules.  The pullbacks solve the
# adjoint system A λ = mask(QQ'(ū)) and pull back the whole residual
# rhs - lhs(ν)(u) (src/adjoint.jl:13-16):
#  - ν: the per-local-copy gradient -G:(grad λ)(grad u) (sem_adjoint_grad);
#  - the right-hand side: mult .* λ.  Fields are local (a global node is stored
#    once per element that holds it) and the cotangents of AD sum over local
#    entries, so an assembled field's cotangent is the global adjoint spread
#    over its copies: a right-hand side mask(QQ'(B f)) then pulls back to
#    B .* λ at f, which central differences in f reproduce.
function varcoef_solve(ν::CuArray{Float64,2}, b::CuArray{Float64,2}, msh::Mesh, bc::Vector{Char};
                       tol=1e-10, k=0.0, precision=SEM_F64_DF)
    set_bc!(msh, bc)
    x = similar(b)
    o = Ref(PcgOpts(1.0, pointer(ν), k, 1, precision, tol, 0, 1e-4, 6, 0, 0, 0))
    info = Ref(SolveInfo())
    check(ccall((:sem_pcg, libsem), Cint,
                (Ptr{Cvoid}, Ref{PcgOpts}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ref{SolveInfo}, Ptr{Cvoid}),
                handle(msh), o, pointer(b), pointer(x), info, stream()))
    return x
end

function adjoint_state(ū, ν, msh::Mesh, bc::Vector{Char}; kw...)
    rhs = gatherScatter(mask(CuArray{Float64,2}(ChainRulesCore.unthunk(ū)),
                             CuArray(Float64.(generateMask(bc, msh)))), msh)
    return varcoef_solve(ν, rhs, msh, bc; kw...)
end

function adjoint_grad(λ::CuArray{Float64,2}, u::CuArray{Float64,2}, msh::Mesh)
    g = similar(u)
    check(ccall((:sem_adjoint_grad, libsem), Cint,
                (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cuint, Ptr{Cvoid}),
                handle(msh), pointer(λ), pointer(u), pointer(g), 0, stream()))
    return g
end

function axpby(α, x::CuArray{Float64,2}, β, y::CuArray{Float64,2})
    out = similar(x)
    check(ccall((:sem_axpby, libsem), Cint,
                (Cdouble, CuPtr{Cdouble}, Cdouble, CuPtr{Cdouble}, CuPtr{Cdouble}, Int64, Ptr{Cvoid}),
                α, pointer(x), β, pointer(y), pointer(out), length(x), stream()))
    return out
end

function ChainRulesCore.rrule(::typeof(varcoef_solve), ν::CuArray{Float64,2}, b::CuArray{Float64,2},
                              msh::Mesh, bc::Vector{Char}; kw...)
    u = varcoef_solve(ν, b, msh, bc; kw...)
    function varcoef_solve_pullback(ū)
        λ = adjoint_state(ū, ν, msh, bc; kw...)
        b̄ = mask(λ, CuArray(msh.mult))
        return ChainRulesCore.NoTangent(), adjoint_grad(λ, u, msh), b̄, ChainRulesCore.NoTangent(),
               ChainRulesCore.NoTangent()
    end
    return u, varcoef_solve_pullback
end

# ---- linsolve(a,problem,solver) (src/adjoint.jl:5-24) on CuArrays.
# problem(a) returns (lhs, rhs): lhs the G-folded operator mask(QQ'(D'(a G)D + k B))
# of `msh` under `bc`, rhs = problem.rhs(a) (any differentiable function of a
# returning a local CuArray) or a fixed field; solver(lhs, rhs, adjoint) is
# Jacobi PCG on the device (the operator is symmetric, so the adjoint solve is
# the same solve).  Other problem or solver types have no device path.
struct VarCoefProblem
    msh::Mesh
    bc::Vector{Char}
    rhs::Any
    k::Float64
end
VarCoefProblem(msh::Mesh, bc::Vector{Char}, rhs; k=0.0) = VarCoefProblem(msh, bc, rhs, Float64(k))

struct VarCoefLHS
    msh::Mesh
    bc::Vector{Char}
    a::CuArray{Float64,2}
    k::Float64
end
(p::VarCoefProblem)(a::CuArray{Float64,2}) =
    (VarCoefLHS(p.msh, p.bc, a, p.k), p.rhs isa Function ? p.rhs(a) : p.rhs)

struct PcgSolver
    tol::Float64
    precision::Cint
end
PcgSolver(; tol=1e-10, precision=SEM_F64_DF) = PcgSolver(tol, precision)
(s::PcgSolver)(lhs::VarCoefLHS, rhs::CuArray{Float64,2}, adjoint::Bool) =
    varcoef_solve(lhs.a, rhs, lhs.msh, lhs.bc; tol=s.tol, k=lhs.k, precision=s.precision)

function linsolve(a::CuArray{Float64,2}, problem::VarCoefProblem, solver::PcgSolver)
    lhs, rhs = problem(a)
    return solver(lhs, rhs, false)
end
linsolve(a::CuArray, problem, solver) =
    throw(ArgumentError("linsolve on CuArrays takes a SEMB200.VarCoefProblem and a SEMB200.PcgSolver"))

function ChainRulesCore.rrule(config::ChainRulesCore.RuleConfig{>:ChainRulesCore.HasReverseMode},
                              ::typeof(linsolve), a::CuArray{Float64,2}, problem::VarCoefProblem,
                              solver::PcgSolver)
    lhs = VarCoefLHS(problem.msh, problem.bc, a, problem.k)
    rhs, rhs_back = problem.rhs isa Function ?
        ChainRulesCore.rrule_via_ad(config, problem.rhs, a) : (problem.rhs, nothing)
    u = solver(lhs, rhs, false)
    kw = (tol=solver.tol, k=problem.k, precision=solver.precision)
    function linsolve_pullback(ū)
        λ = adjoint_state(ū, a, problem.msh, problem.bc; kw...)
        ā = adjoint_grad(λ, u, problem.msh)                    # -λ' d(lhs(a) u)/da
        if rhs_back !== nothing
            r̄ = ChainRulesCore.unthunk(rhs_back(mask(λ, CuArray(problem.msh.mult)))[2])
            ā = axpby(1.0, ā, 1.0, CuArray{Float64,2}(r̄))     # + λ' d rhs(a)/da
        end
        return ChainRulesCore.NoTangent(), ā, ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent()
    end
    return u, linsolve_pullback
end

end # module
