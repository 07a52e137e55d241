# HelmholtzGB300: Julia binding of the helmgpu C ABI (include/helmgpu.h).
#
# Drop-in for the shifted-Laplacian multigrid path of Helmholtz.jl: the same
# names and argument orders as src/ShiftedLaplacianMultigridSolver.jl and
# src/GetHelmholtz.jl, with the solve running on one GB300 through ccall.
# Matrices handed in by callers (ShiftedHT) are not read; the library
# rebuilds the operator matrix-free from HelmholtzParam.
#
# Load with
#     ENV["HELMGPU_LIB"] = "/path/to/libhelmgpu.so"   # optional
#     include("HelmholtzGB300.jl"); using .HelmholtzGB300
# Requires jInv (RegularMesh) and Multigrid (MGparam) as Helmholtz.jl does.
module HelmholtzGB300

using LinearAlgebra
using SparseArrays
using jInv.Mesh
import jInv.LinearSolvers: AbstractSolver, solveLinearSystem, solveLinearSystem!
import jInv.Utils.clear!
using Multigrid: MGparam

export HelmholtzParam, ShiftedLaplacianMultigridSolver, getShiftedLaplacianMultigridSolver, solveLinearSystem,
       solveLinearSystem!, copySolver, clear!, getMaximalFrequency, getABL, getSommerfeldBC,
       getAcousticPointSource, getHelmholtzFun, HzApply, applyNoAlloc!,
       helmgpuVersion, columnStats, setCudaGraph!, setProfile!, kernelTimes, resetKernelTimes!, tuneInfo,
       learnedStats,
       CoarseNet, netWeights, setNetWeights!, netForward, netGradient, netTrain!, collectPairs!, attachNet!,
       saveNet, loadNet!

const libhelmgpu = get(ENV, "HELMGPU_LIB", joinpath(@__DIR__, "..", "libhelmgpu.so"))

# ---- C structs (field order and types of include/helmgpu.h) -----------------
struct HzProblem
    dim::Int32
    n::NTuple{3,Int64}
    h::NTuple{3,Float64}
    omega_re::Float64
    omega_im::Float64
    m::Ptr{Float64}
    gamma::Ptr{Float64}
    neumann_on_top::Int32
    sommerfeld::Int32
    order_neumann_bc::Int32
end

mutable struct HzOptions
    levels::Int32
    max_outer::Int32
    rel_tol::Float64
    relax_pre::Int32
    relax_post::Int32
    relax_param::Float64
    cycle::Int32
    krylov::Int32
    inner::Int32
    shift::Float64
    precision::Int32
    coarse_op::Int32
    verbose::Int32
    profile::Int32
    device::Int32
    outer_arith::Int32
    cuda_graph::Int32
    autotune::Int32
    relax_type::Int32
    relax_from::Int32
    reserved::NTuple{2,Int32}
end
HzOptions() = HzOptions(0, 0, 0.0, 0, 0, 0.0, 0, 0, 0, 0.0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, ntuple(_ -> Int32(0), 2))

mutable struct HzStats
    outer::Int32
    n_prec::Int32
    max_col_iters::Int32
    converged_cols::Int32
    max_relres::Float64
    setup_time::Float64
    solve_time::Float64
    kernel_launches::Int64
    h2d_bytes::Int64
    d2h_bytes::Int64
end
HzStats() = HzStats(0, 0, 0, 0, 0.0, 0.0, 0.0, 0, 0, 0)

const HZ_MEM_HOST = Int32(0)
const HZ_PREC_FP64 = Int32(0)
const HZ_PREC_MIXED = Int32(1)
const HZ_OP_H = Int32(0)
const HZ_MEM_DEVICE = Int32(1)
const HZ_OUTER_FP64 = Int32(0)
const HZ_OUTER_EMULATED = Int32(1)
const HZ_KRYLOV_FGMRES = Int32(0)
const HZ_KRYLOV_BICGSTAB = Int32(1)
const HZ_COARSE_GALERKIN = Int32(0)
const HZ_COARSE_REDISCRETIZE = Int32(1)
const HZ_RELAX_JAC = Int32(0)
const HZ_RELAX_JAC_GMRES = Int32(1)
const HZ_NET_CONV_WARP_MMA = Int32(0)
const HZ_NET_CONV_TCGEN05 = Int32(1)
const HZ_NET_CONV_AUTO = Int32(2)

lasterror(h::Ptr{Cvoid}) = unsafe_string(ccall((:hz_last_error, libhelmgpu), Cstring, (Ptr{Cvoid},), h))
function check(st::Integer, h::Ptr{Cvoid} = C_NULL)
    st < 0 && throw(ErrorException("helmgpu error $st: " * lasterror(h)))
    return st
end

# ---- Helmholtz problem ---------------------------------------------------------
mutable struct HelmholtzParam      # src/Helmholtz.jl:13-20
    Mesh::RegularMesh
    gamma::Array{Float64}
    m::Array{Float64}
    omega::Union{Float64,ComplexF64}
    NeumannOnTop::Bool
    Sommerfeld::Bool
end

function hzproblem(p::HelmholtzParam, order::Int = 2)
    M = p.Mesh
    n = ntuple(i -> i <= M.dim ? Int64(M.n[i]) : Int64(0), 3)
    h = ntuple(i -> i <= M.dim ? Float64(M.h[i]) : 0.0, 3)
    w = ComplexF64(p.omega)
    return HzProblem(Int32(M.dim), n, h, real(w), imag(w), pointer(p.m), pointer(p.gamma),
                     Int32(p.NeumannOnTop), Int32(p.Sommerfeld), Int32(order))
end

getMaximalFrequency(m::Array{Float64}, M::RegularMesh) =
    ccall((:hz_max_frequency, libhelmgpu), Float64, (Ptr{Float64}, Int64, Ptr{Float64}, Int32),
          m, length(m), collect(Float64, M.h), Int32(M.dim))

function getABL(n::Array{Int64}, NeumannAtFirstDim::Bool, ABLpad::Array{Int64}, ABLamp::Float64)
    g = zeros(Float64, tuple(n...))
    check(ccall((:hz_abl, libhelmgpu), Cint, (Int32, Ptr{Int64}, Int32, Ptr{Int64}, Float64, Ptr{Float64}),
                Int32(length(n)), n, Int32(NeumannAtFirstDim), ABLpad, ABLamp, g))
    return g
end

function getSommerfeldBC(Msh::RegularMesh, mNodal::Array{Float64}, omega::Float64, NeumannOnTop::Bool,
                         orderNeumannBC = 2)
    S = zeros(ComplexF64, tuple((Msh.n .+ 1)...))
    check(ccall((:hz_sommerfeld, libhelmgpu), Cint,
                (Int32, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Int32, Ptr{ComplexF64}),
                Int32(Msh.dim), collect(Int64, Msh.n), collect(Float64, Msh.h), mNodal, omega,
                Int32(NeumannOnTop), Int32(orderNeumannBC), S))
    return S
end

function getAcousticPointSource(Minv::RegularMesh, TYPE, src = nothing)
    if src === nothing
        src = Minv.dim == 3 ? [div(Minv.n[1] + 1, 2); div(Minv.n[2] + 1, 2); 1] : [div(Minv.n[1] + 1, 2); 1]
    end
    q = zeros(ComplexF64, tuple((Minv.n .+ 1)...))
    check(ccall((:hz_point_source, libhelmgpu), Cint, (Int32, Ptr{Int64}, Ptr{Float64}, Ptr{Int64}, Ptr{ComplexF64}),
                Int32(Minv.dim), collect(Int64, Minv.n), collect(Float64, Minv.h), collect(Int64, src), q))
    return convert(Array{TYPE}, q), src
end

# ---- solver ----------------------------------------------------------------------
mutable struct ShiftedLaplacianMultigridSolver <: AbstractSolver   # src/ShiftedLaplacianMultigridSolver.jl:4-15
    helmParam::HelmholtzParam
    MG::MGparam
    shift::Array{Float64}
    Krylov::String
    inner::Int64
    doClear::Int64
    verbose::Bool
    setupTime::Real
    nPrec::Int
    solveTime::Real
    precision::Int32            # HZ_PREC_FP64 (plain) or HZ_PREC_MIXED
    outerArith::Int32           # HZ_OUTER_FP64 or HZ_OUTER_EMULATED (mixed form only)
    coarseOp::Int32             # HZ_COARSE_GALERKIN or HZ_COARSE_REDISCRETIZE
    relaxFrom::Int32            # relaxType "Jac-GMRES": first level smoothed by GMRES steps
    handle::Ptr{Cvoid}
    net::Any                    # attached CoarseNet (or nothing), its level and stagnation ratio
    netLevel::Int32
    netStag::Float64
end

function getShiftedLaplacianMultigridSolver(helmParam::HelmholtzParam, MG::MGparam, shift::Array{Float64},
                                            Krylov::String = "BiCGSTAB", inner::Int64 = 5, verbose::Bool = false;
                                            precision::Int32 = HZ_PREC_FP64, outerArith::Int32 = HZ_OUTER_FP64,
                                            coarseOp::Int32 = HZ_COARSE_GALERKIN, relaxFrom::Int32 = Int32(0))
    s = ShiftedLaplacianMultigridSolver(helmParam, MG, shift, Krylov, inner, 0, verbose, 0.0, 0, 0.0, precision,
                                        outerArith, coarseOp, relaxFrom, C_NULL, nothing, Int32(0), 0.95)
    finalizer(release!, s)
    return s
end
getShiftedLaplacianMultigridSolver(helmParam::HelmholtzParam, MG::MGparam, shift::Float64, Krylov::String = "BiCGSTAB",
                                   inner::Int64 = 5, verbose::Bool = false; kw...) =
    getShiftedLaplacianMultigridSolver(helmParam, MG, ones(MG.levels) * shift, Krylov, inner, verbose; kw...)

function release!(s::ShiftedLaplacianMultigridSolver)
    s.handle != C_NULL && ccall((:hz_destroy, libhelmgpu), Cint, (Ptr{Cvoid},), s.handle)
    s.handle = C_NULL
    return nothing
end

function options(s::ShiftedLaplacianMultigridSolver)
    MG = s.MG
    MG.relaxType in ("Jac", "Jac-GMRES") ||
        throw(ArgumentError("relaxType $(MG.relaxType): \"Jac\" and \"Jac-GMRES\" are built"))
    MG.cycleType in ('V', 'W', 'K') ||
        throw(ArgumentError("cycleType $(MG.cycleType): only 'V', 'W' and 'K' are built"))
    s.Krylov in ("GMRES", "BiCGSTAB") ||
        throw(ArgumentError("Krylov $(s.Krylov): \"GMRES\" (FGMRES) and \"BiCGSTAB\" are built"))
    o = HzOptions()
    ccall((:hz_default_options, libhelmgpu), Cvoid, (Ref{HzOptions},), o)
    o.levels = MG.levels
    o.max_outer = MG.maxOuterIter
    o.rel_tol = MG.relativeTol
    o.relax_pre = MG.relaxPre
    o.relax_post = MG.relaxPost
    o.relax_param = MG.relaxParam
    o.cycle = Int32(MG.cycleType)
    o.inner = s.inner
    o.shift = s.shift[1]
    o.precision = s.precision
    o.outer_arith = s.outerArith
    o.coarse_op = s.coarseOp
    o.relax_type = MG.relaxType == "Jac-GMRES" ? HZ_RELAX_JAC_GMRES : HZ_RELAX_JAC
    o.relax_from = s.relaxFrom
    o.krylov = s.Krylov == "BiCGSTAB" ? HZ_KRYLOV_BICGSTAB : HZ_KRYLOV_FGMRES
    o.verbose = Int32(s.verbose)
    return o
end

function ensure_handle!(s::ShiftedLaplacianMultigridSolver)
    s.handle != C_NULL && return s.handle
    prob = hzproblem(s.helmParam)
    o = options(s)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve s begin
        check(ccall((:hz_create, libhelmgpu), Cint, (Ref{HzProblem}, Ref{HzOptions}, Ref{Ptr{Cvoid}}), prob, o, h))
    end
    s.handle = h[]
    s.net === nothing || attach_handle!(s)
    return s.handle
end

# src/ShiftedLaplacianMultigridSolver.jl:33-102
function solveLinearSystem(ShiftedHT, B, param::ShiftedLaplacianMultigridSolver, doTranspose::Int64 = 0)
    if size(B, 2) == 1
        B = vec(B)
    end
    if param.doClear == 1
        clear!(param)
    end
    if norm(B) == 0.0
        return zeros(eltype(B), size(B)), param
    end
    h = ensure_handle!(param)
    Bc = convert(Array{ComplexF64}, B)
    X = similar(Bc)
    st = HzStats()
    code = ccall((:hz_solve, libhelmgpu), Cint,
                 (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Ref{HzStats}),
                 h, Bc, X, size(Bc, 1), Int32(size(Bc, 2)), Int32(doTranspose), HZ_MEM_HOST, st)
    check(code, h)
    param.setupTime = st.setup_time
    param.solveTime = st.solve_time
    param.nPrec += st.outer
    if code > 0
        println("WARNING: MG solver reached maximum iterations without convergence")
    end
    return X, param
end

function solveLinearSystem!(A, B, X, param::ShiftedLaplacianMultigridSolver, doTranspose::Int64 = 0)
    Y, param = solveLinearSystem(A, B, param, doTranspose)
    X .= reshape(Y, size(X))
    return X, param
end

function copySolver(s::ShiftedLaplacianMultigridSolver)   # src/ShiftedLaplacianMultigridSolver.jl:18-22
    return getShiftedLaplacianMultigridSolver(s.helmParam, s.MG, s.shift, s.Krylov, s.inner, s.verbose;
                                              precision = s.precision, outerArith = s.outerArith,
                                              coarseOp = s.coarseOp, relaxFrom = s.relaxFrom)
end

function clear!(s::ShiftedLaplacianMultigridSolver)        # src/ShiftedLaplacianMultigridSolver.jl:105-109
    s.handle != C_NULL && check(ccall((:hz_clear, libhelmgpu), Cint, (Ptr{Cvoid},), s.handle), s.handle)
    s.doClear = 0
    return nothing
end

# getHelmholtzFun (src/GetHelmholtz.jl:85-95): y = H x on the GPU.  The sparse
# ShiftedHT / ShiftMat arguments of the reference are replaced by the solver
# that owns the problem; transpose = 1 gives H^H x (the doTranspose pair).
struct HzApply
    s::ShiftedLaplacianMultigridSolver
    transpose::Int32
end
function (f::HzApply)(x::AbstractVecOrMat)
    h = ensure_handle!(f.s)
    xc = convert(Array{ComplexF64}, x)
    y = similar(xc)
    check(ccall((:hz_apply, libhelmgpu), Cint,
                (Ptr{Cvoid}, Int32, Int32, Ptr{ComplexF64}, Ptr{ComplexF64}, Int64, Int32, Int32),
                h, HZ_OP_H, f.transpose, xc, y, size(xc, 1), Int32(size(xc, 2)), HZ_MEM_HOST), h)
    return y
end
getHelmholtzFun(s::ShiftedLaplacianMultigridSolver, transpose::Integer = 0) = HzApply(s, Int32(transpose))

# Y = H X on DEVICE arrays (e.g. CUDA.jl CuArray pointers, n x nrhs complex FP64)
# without any GPU memory allocation; the caller's writes of X must be complete
# (synchronised) before the call.
function applyNoAlloc!(s::ShiftedLaplacianMultigridSolver, X::Ptr{ComplexF64}, Y::Ptr{ComplexF64}, n::Integer,
                       nrhs::Integer, transpose::Integer = 0)
    h = ensure_handle!(s)
    check(ccall((:hz_apply_noalloc, libhelmgpu), Cint,
                (Ptr{Cvoid}, Int32, Int32, Ptr{ComplexF64}, Ptr{ComplexF64}, Int64, Int32),
                h, HZ_OP_H, Int32(transpose), X, Y, Int64(n), Int32(nrhs)), h)
    return Y
end

# ---- diagnostics (no counterpart in the reference) --------------------------------
helmgpuVersion() = Int(ccall((:hz_version, libhelmgpu), Int32, ()))

# per-column relative residuals and iteration counts of the last solve of s
function columnStats(s::ShiftedLaplacianMultigridSolver, nrhs::Integer)
    s.handle == C_NULL && throw(ArgumentError("the solver has not solved yet"))
    rr = zeros(Float64, nrhs)
    it = zeros(Int32, nrhs)
    check(ccall((:hz_column_stats, libhelmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Int32}, Int32),
                s.handle, rr, it, Int32(nrhs)), s.handle)
    return rr, it
end

# replay the preconditioner's cycles from CUDA graphs (true, the default) or launch them one by one
setCudaGraph!(s::ShiftedLaplacianMultigridSolver, on::Bool) =
    check(ccall((:hz_set_cuda_graph, libhelmgpu), Cint, (Ptr{Cvoid}, Int32), ensure_handle!(s), Int32(on)),
          s.handle)
# per-launch CUDA-event timing of the kernels (for kernelTimes)
setProfile!(s::ShiftedLaplacianMultigridSolver, on::Bool) =
    check(ccall((:hz_set_profile, libhelmgpu), Cint, (Ptr{Cvoid}, Int32), ensure_handle!(s), Int32(on)), s.handle)

# the handle's launch table: (name, launches, timed launches, total ms, algorithmic bytes, algorithmic flops)
function kernelTimes(s::ShiftedLaplacianMultigridSolver)
    h = ensure_handle!(s)
    n = ccall((:hz_kernel_times, libhelmgpu), Cint,
              (Ptr{Cvoid}, Int32, Ptr{UInt8}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
              h, Int32(-1), C_NULL, Int32(0), C_NULL, C_NULL, C_NULL, C_NULL)
    check(n, h)
    rows = Vector{NamedTuple}()
    for i in 0:n-1
        name = zeros(UInt8, 64)
        la, lt, ms, by, fl = Ref{Int64}(0), Ref{Int64}(0), Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{Float64}(0.0)
        check(ccall((:hz_kernel_times, libhelmgpu), Cint,
                    (Ptr{Cvoid}, Int32, Ptr{UInt8}, Int32, Ref{Int64}, Ref{Int64}, Ref{Float64}, Ref{Float64}),
                    h, Int32(i), name, Int32(64), la, lt, ms, by), h)
        check(ccall((:hz_kernel_flops, libhelmgpu), Cint, (Ptr{Cvoid}, Int32, Ref{Float64}), h, Int32(i), fl), h)
        push!(rows, (name = unsafe_string(pointer(name)), launches = la[], timed = lt[], ms = ms[],
                     bytes = by[], flops = fl[]))
    end
    return rows
end
resetKernelTimes!(s::ShiftedLaplacianMultigridSolver) =
    check(ccall((:hz_reset_kernel_times, libhelmgpu), Cint, (Ptr{Cvoid},), ensure_handle!(s)), s.handle)
# launch shapes the autotuner chose (CTAs per launch of the fine and the Galerkin stencils)
function tuneInfo(s::ShiftedLaplacianMultigridSolver)
    f, r = Ref{Int32}(0), Ref{Int32}(0)
    st = check(ccall((:hz_tune_info, libhelmgpu), Cint, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}), ensure_handle!(s), f, r),
               s.handle)
    return st == 0 ? (fine = Int(f[]), rap = Int(r[])) : nothing
end
# network applications and fallbacks to the plain cycle in the solves of s
function learnedStats(s::ShiftedLaplacianMultigridSolver)
    c, f = Ref{Int64}(0), Ref{Int32}(0)
    s.handle == C_NULL && return (calls = 0, fallbacks = 0)
    check(ccall((:hz_learned_stats, libhelmgpu), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int32}), s.handle, c, f), s.handle)
    return (calls = Int(c[]), fallbacks = Int(f[]))
end

# ---- learned coarse-grid correction (no counterpart in the reference) ------------
# Arrays are Julia column-major (4, nx, ny, batch) for inputs and (2, nx, ny, batch)
# for targets / outputs (Float32): the C layout [batch][nx*ny][channels].
mutable struct CoarseNet
    ptr::Ptr{Cvoid}
end
function CoarseNet(seed::Integer = 0, device::Integer = 0)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hz_net_create, libhelmgpu), Cint, (Int32, Int32, Ref{Ptr{Cvoid}}), seed, device, p))
    net = CoarseNet(p[])
    finalizer(n -> (n.ptr != C_NULL && ccall((:hz_net_destroy, libhelmgpu), Cint, (Ptr{Cvoid},), n.ptr);
                    n.ptr = C_NULL), net)
    return net
end
function netWeights(net::CoarseNet)
    w = Vector{Float32}(undef, ccall((:hz_net_num_params, libhelmgpu), Int64, ()))
    check(ccall((:hz_net_get_weights, libhelmgpu), Cint, (Ptr{Cvoid}, Ptr{Float32}), net.ptr, w))
    return w
end
setNetWeights!(net::CoarseNet, w::Vector{Float32}) =
    check(ccall((:hz_net_set_weights, libhelmgpu), Cint, (Ptr{Cvoid}, Ptr{Float32}), net.ptr, w))
function netForward(net::CoarseNet, x::Array{Float32,4})
    _, nx, ny, b = size(x)
    y = Array{Float32}(undef, 2, nx, ny, b)
    check(ccall((:hz_net_forward, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int32, Int32),
                net.ptr, x, y, nx, ny, Int32(b), HZ_MEM_HOST))
    return y
end
function netGradient(net::CoarseNet, x::Array{Float32,4}, t::Array{Float32,4})
    _, nx, ny, b = size(x)
    g = similar(netWeights(net))
    loss = Ref{Float64}(0.0)
    check(ccall((:hz_net_gradient, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int32, Int32, Ref{Float64}, Ptr{Float32}),
                net.ptr, x, t, nx, ny, Int32(b), HZ_MEM_HOST, loss, g))
    return loss[], g
end
# x, t: DEVICE pointers (e.g. from CUDA.jl CuArrays) to npairs pairs
function netTrain!(net::CoarseNet, x::Ptr{Float32}, t::Ptr{Float32}, nx::Integer, ny::Integer, npairs::Integer;
                   batch::Integer = 32, epochs::Integer = 20, lr::Float64 = 2e-3, seed::Integer = 0)
    hist = zeros(Float64, epochs)
    check(ccall((:hz_net_train, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int64, Int32, Int32, Float64, Int32,
                 Ptr{Float64}),
                net.ptr, x, t, nx, ny, npairs, Int32(batch), Int32(epochs), lr, Int32(seed), hist))
    return hist
end
# solves with the FP64 solver s while recording the pairs of `level` into the DEVICE
# arrays x (4 x nx x ny x maxPairs) and t (2 x nx x ny x maxPairs); returns (count, plainErr, X)
function collectPairs!(s::ShiftedLaplacianMultigridSolver, B::AbstractVecOrMat, level::Integer, maxPairs::Integer,
                       x::Ptr{Float32}, t::Ptr{Float32}; sweeps::Integer = 2)
    h = ensure_handle!(s)
    Bc = convert(Matrix{ComplexF64}, reshape(B, size(B, 1), :))
    X = similar(Bc)
    pe = zeros(Float64, maxPairs)
    rr = Ref{Float64}(0.0)
    cnt = Ref{Int64}(0)
    check(ccall((:hz_collect_pairs, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Int32, Int64,
                 Ptr{Float32}, Ptr{Float32}, Ptr{Float64}, Ref{Float64}, Ref{Int64}),
                h, Bc, X, size(Bc, 1), Int32(size(Bc, 2)), HZ_MEM_HOST, Int32(level), Int32(sweeps), maxPairs,
                x, t, pe, rr, cnt), h)
    return cnt[], pe[1:cnt[]], X
end
# The 3D network (three grid levels, 8-16-32 channels, 3x3x3 convolutions): arrays
# (4, nx, ny, nz, batch) and (2, nx, ny, nz, batch); node counts 4k+1.  Weights,
# files, profiling and attachNet! take it like the 2D one.
function CoarseNet3D(seed::Integer = 0, device::Integer = 0)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hz_net3d_create, libhelmgpu), Cint, (Int32, Int32, Ref{Ptr{Cvoid}}), seed, device, p))
    net = CoarseNet(p[])
    finalizer(n -> (n.ptr != C_NULL && ccall((:hz_net_destroy, libhelmgpu), Cint, (Ptr{Cvoid},), n.ptr);
                    n.ptr = C_NULL), net)
    return net
end
netDim(net::CoarseNet) = Int(ccall((:hz_net_dim, libhelmgpu), Cint, (Ptr{Cvoid},), net.ptr))
# convolution kernels of a network: HZ_NET_CONV_WARP_MMA, HZ_NET_CONV_TCGEN05 or
# HZ_NET_CONV_AUTO (the default: per layer the faster)
setNetConvPath!(net::CoarseNet, path::Integer) =
    check(ccall((:hz_net_set_conv_path, libhelmgpu), Cint, (Ptr{Cvoid}, Int32), net.ptr, Int32(path)))
function netWeights3D(net::CoarseNet)
    w = Vector{Float32}(undef, ccall((:hz_net3d_num_params, libhelmgpu), Int64, ()))
    check(ccall((:hz_net_get_weights, libhelmgpu), Cint, (Ptr{Cvoid}, Ptr{Float32}), net.ptr, w))
    return w
end
function netForward(net::CoarseNet, x::Array{Float32,5})
    _, nx, ny, nz, b = size(x)
    y = Array{Float32}(undef, 2, nx, ny, nz, b)
    check(ccall((:hz_net3d_forward, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int64, Int32, Int32),
                net.ptr, x, y, nx, ny, nz, Int32(b), HZ_MEM_HOST))
    return y
end
function netGradient(net::CoarseNet, x::Array{Float32,5}, t::Array{Float32,5})
    _, nx, ny, nz, b = size(x)
    g = netWeights3D(net)
    loss = Ref{Float64}(0.0)
    check(ccall((:hz_net3d_gradient, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int64, Int32, Int32, Ref{Float64},
                 Ptr{Float32}),
                net.ptr, x, t, nx, ny, nz, Int32(b), HZ_MEM_HOST, loss, g))
    return loss[], g
end
function netTrain3D!(net::CoarseNet, x::Ptr{Float32}, t::Ptr{Float32}, nx::Integer, ny::Integer, nz::Integer,
                     npairs::Integer; batch::Integer = 8, epochs::Integer = 20, lr::Float64 = 2e-3,
                     seed::Integer = 0)
    hist = zeros(Float64, epochs)
    check(ccall((:hz_net3d_train, libhelmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Int64, Int64, Int64, Int64, Int32, Int32, Float64, Int32,
                 Ptr{Float64}),
                net.ptr, x, t, nx, ny, nz, npairs, Int32(batch), Int32(epochs), lr, Int32(seed), hist))
    return hist
end
# versioned file of the weights and the Adam state; training resumes from a loaded file
saveNet(net::CoarseNet, path::AbstractString) =
    check(ccall((:hz_net_save, libhelmgpu), Cint, (Ptr{Cvoid}, Cstring), net.ptr, path))
loadNet!(net::CoarseNet, path::AbstractString) =
    check(ccall((:hz_net_load, libhelmgpu), Cint, (Ptr{Cvoid}, Cstring), net.ptr, path))
# use net for the coarse-grid correction of `level` in the later solves of s (FGMRES only);
# net = nothing detaches
function attachNet!(s::ShiftedLaplacianMultigridSolver, net, level::Integer = 2, stagRatio::Float64 = 0.95)
    s.net = net
    s.netLevel = Int32(level)
    s.netStag = stagRatio
    s.handle != C_NULL && attach_handle!(s)
    return s
end
function attach_handle!(s::ShiftedLaplacianMultigridSolver)
    p = s.net === nothing ? C_NULL : s.net.ptr
    check(ccall((:hz_attach_net, libhelmgpu), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Float64),
                s.handle, p, s.netLevel, s.netStag), s.handle)
end

end # module
