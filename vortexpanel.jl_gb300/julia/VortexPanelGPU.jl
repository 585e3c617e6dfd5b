"""
    VortexPanelGPU

Julia bindings of libvortexpanel_gpu.so (the C ABI of include/vortexpanel_gpu.h) for VortexPanel.jl: the Galerkin hot
path on one GB300 with the reference's signatures. Included from VortexPanel.jl as `src/gpu/VortexPanelGPU.jl` (it
uses the package's Geometry, DOFMap, Assembly, Elements and FreeWake modules); the library path comes from
`ENV["VORTEXPANEL_GPU_LIB"]`.

  assemble(g, dm, els, σ, V∞; opts, external, wake, precision)   src/assembly/assemble.jl:377-447
  factorize_galerkin(dm, A; W, precision)                         src/assembly/solve.jl:81-87
  solve_galerkin(F, b), solve_galerkin(dm, A, b; W)              src/assembly/solve.jl:51-59,95-99
  consistency(dm, A, b; W)                                        src/assembly/solve.jl:111-115
  pressure_force, kutta_joukowski_force, trefftz_drag             src/post/forces.jl:11-81
  GPUFreeWakeSim, step!, run!                                     src/freewake/step.jl:35-216
  ChainRulesCore.rrule(wing_loads, x, α)                          the adjoint (vp_solve_transposed, vp_adjoint)

A stays on the GPU as a `DeviceSystem`; `Matrix(A)` copies it to the host for the reference's callers that read A
(`reduce_system` on the host, plots). Arrays cross the boundary as the ABI wants them: a 3 × n coordinate matrix
(`reduce(hcat, g.x)`) is the ABI's n × 3 row-major layout, indices go in 0-based.
"""
module VortexPanelGPU

using LinearAlgebra, SparseArrays, StaticArrays
using ChainRulesCore
using ..Geometry: SurfaceGeometry
using ..DOFMap: DOFMapping, wake_rows
using ..Elements: build_elements, point, triangle_rule
using ..Wake: te_panel
using ..Assembly
using ..Assembly: AssemblyOptions
using ..FreeWake
using ..FreeWake: FreeWakeOptions

const LIB = get(ENV, "VORTEXPANEL_GPU_LIB", "libvortexpanel_gpu.so")

# ---- structures of the ABI --------------------------------------------------------------------------------------------

# vp_assembly_options: test 0 hat, 1 onering, 2 dual; precision 0 FP64, 1 mixed
struct VpOptions
    test::Cint
    far_ratio::Cdouble
    far_points::Cint
    near_points::Cint
    near_ratio::Cdouble
    near_depth::Cint
    touch_levels::Cint
    touch_ratio::Cdouble
    touch_order::Cint
    corner_angle::Cdouble
    contact_rel::Cdouble
    kernel_far::Cdouble
    precision::Cint
end

VpOptions(o::AssemblyOptions; precision::Symbol=:fp64) = VpOptions(Cint(findfirst(==(o.test), (:hat, :onering, :dual)) - 1),
    o.far_ratio, o.far_points, o.near_points, o.near_ratio, o.near_depth, o.touch_levels, o.touch_ratio, o.touch_order,
    o.corner_angle, o.contact_rel, o.kernel_far, precision === :mixed ? Cint(1) : Cint(0))

# vp_assembly_stats
struct VpStats
    pairs::NTuple{6,Clonglong}
    points::NTuple{6,Clonglong}
    time_ms::Cdouble
    points_fp64::Clonglong
end

# ---- context and errors ---------------------------------------------------------------------------------------------

mutable struct Context
    h::Ptr{Cvoid}
end

function Context(device::Integer=0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(C_NULL, ccall((:vp_ctx_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), device, h))
    c = Context(h[])
    finalizer(c -> ccall((:vp_ctx_destroy, LIB), Cvoid, (Ptr{Cvoid},), c.h), c)
end

const DEFAULT = Ref{Union{Nothing,Context}}(nothing)
default_context() = something(DEFAULT[], (DEFAULT[] = Context(0)))

"""The reference's exceptions for the library's status codes"""
function check(ctx, status::Cint)
    status == 0 && return nothing
    msg = ctx == C_NULL ? "" : unsafe_string(ccall((:vp_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx))
    status in (1, 2) && throw(ArgumentError(msg))            # VP_ERR_ARG, VP_ERR_DEGENERATE
    status == 3 && throw(LinearAlgebra.SingularException(0))  # VP_ERR_SINGULAR
    error("libvortexpanel_gpu status $status: $msg")
end

flat(v::AbstractVector{<:SVector{3}}) = collect(Cdouble, reduce(vcat, v))   # n x 3 row-major
test_weights(test, λ) = Assembly.test_weights(test, λ)                      # assemble.jl:52-58

"""the 1-based body of every unknown (0 for none), from the DOF map's unknowns per body"""
function q_body(dm::DOFMapping)
    qb = zeros(Cint, dm.nq)
    for (b, qs) in enumerate(dm.body_q), q in qs
        qb[q] = b
    end
    return qb
end
idx0(v::AbstractVector) = Cint.(reduce(vcat, collect.(v)) .- 1)           # 0-based, row-major
csr(M::SparseMatrixCSC) = (t = sparse(transpose(M)); (Cint.(t.colptr .- 1), Cint.(t.rowval .- 1), collect(Cdouble, t.nzval)))

# ---- assembly ---------------------------------------------------------------------------------------------------------

mutable struct DeviceSystem <: AbstractMatrix{Cdouble}
    ctx::Context
    h::Ptr{Cvoid}
    nslot::Int
    ncols::Int
end

Base.size(A::DeviceSystem) = (A.nslot, A.ncols)
Base.getindex(A::DeviceSystem, i::Int, j::Int) = rows(A, i:i)[1, j]

"""rows r (a unit range) of A to the host"""
function rows(A::DeviceSystem, r::UnitRange{Int})
    out = Matrix{Cdouble}(undef, A.ncols, length(r))   # row-major rows = columns of the transpose
    check(A.ctx.h, ccall((:vp_system_download_rows, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}),
        A.ctx.h, A.h, first(r) - 1, last(r), out, C_NULL))
    return permutedims(out)
end

"""A as a host Matrix (the reference's assemble returns one, assemble.jl:446)"""
function Base.Matrix(A::DeviceSystem)
    out = Matrix{Cdouble}(undef, A.ncols, A.nslot)
    check(A.ctx.h, ccall((:vp_system_download, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
        A.ctx.h, A.h, out, C_NULL))
    return permutedims(out)
end

function assemble(g::SurfaceGeometry, dm::DOFMapping, els, σ, V∞; opts=AssemblyOptions(), external=nothing,
    wake=nothing, precision::Symbol=:fp64, ctx::Context=default_context())
    o = Ref(VpOptions(opts; precision))
    tp = isempty(g.touch_pairs) ? Cint[0, 0] : idx0(g.touch_pairs)
    nw = wake === nothing ? 0 : length(wake.x)
    wx = wake === nothing ? Cdouble[0] : flat(wake.x)
    wt = wake === nothing || isempty(wake.tris) ? Cint[0, 0, 0] : idx0(wake.tris)
    wf = wake === nothing || isempty(wake.filaments) ? Cint[0, 0] : idx0(wake.filaments)
    nwt = wake === nothing ? 0 : length(wake.tris)
    nf = wake === nothing ? 0 : length(wake.filaments)
    h, st = Ref{Ptr{Cvoid}}(C_NULL), Ref{VpStats}()
    check(ctx.h, ccall((:vp_assemble, LIB), Cint,
        (Ptr{Cvoid}, Ref{VpOptions}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cint}, Cint, Cint, Ptr{Cint}, Ptr{Cdouble},
         Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Ref{Ptr{Cvoid}}, Ref{VpStats}),
        ctx.h, o, length(g.x), flat(g.x), length(g.tris), idx0(g.tris), idx0(dm.corner_slot), dm.nslot,
        length(g.touch_pairs), tp, collect(Cdouble, σ), collect(Cdouble, V∞), nw, wx, nwt, wt, nf, wf, h, st))
    A = DeviceSystem(ctx, h[], dm.nslot, dm.nslot + nw)
    finalizer(a -> ccall((:vp_system_free, LIB), Cvoid, (Ptr{Cvoid},), a.h), A)
    b = Vector{Cdouble}(undef, dm.nslot)
    check(ctx.h, ccall((:vp_system_download, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
        ctx.h, A.h, C_NULL, b))
    if external !== nothing  # the external field's part of b, as the reference adds it (assemble.jl:423-427)
        rule = triangle_rule(7)
        for (t, T) in enumerate(els), (λ, wq) in zip(rule.λ, rule.w)
            un = wq * T.area * dot(external(point(T, λ)), T.n)
            b[collect(dm.corner_slot[t])] .-= un .* test_weights(opts.test, λ)
        end
    end
    return A, b, st[]
end

# vp_assembly_input (vortexpanel_gpu.h): one body of a batch; the arrays it points to are kept alive by the caller
struct VpInput
    nnode::Cint; x::Ptr{Cdouble}; ntri::Cint; tris::Ptr{Cint}; corner_slot::Ptr{Cint}; nslot::Cint
    ntouch::Cint; touch_pairs::Ptr{Cint}; sigma::Ptr{Cdouble}; vinf::Ptr{Cdouble}
    nwnode::Cint; wx::Ptr{Cdouble}; nwtri::Cint; wtris::Ptr{Cint}; nfil::Cint; fil::Ptr{Cint}
end

# assemble for several bodies of uneven sizes in shared launches (vp_assemble_batch); cases: (g, dm, σ, V∞, wake)
function assemble_batch(cases; opts=AssemblyOptions(), precision::Symbol=:fp64, ctx::Context=default_context())
    o = Ref(VpOptions(opts; precision))
    keep = Any[]
    ins = VpInput[]
    for (g, dm, σ, V∞, wake) in cases
        a = (flat(g.x), idx0(g.tris), idx0(dm.corner_slot),
             isempty(g.touch_pairs) ? Cint[0, 0] : idx0(g.touch_pairs), collect(Cdouble, σ), collect(Cdouble, V∞),
             wake === nothing ? Cdouble[0] : flat(wake.x),
             wake === nothing || isempty(wake.tris) ? Cint[0, 0, 0] : idx0(wake.tris),
             wake === nothing || isempty(wake.filaments) ? Cint[0, 0] : idx0(wake.filaments))
        push!(keep, a)
        nw = wake === nothing ? 0 : length(wake.x)
        push!(ins, VpInput(length(g.x), pointer(a[1]), length(g.tris), pointer(a[2]), pointer(a[3]), dm.nslot,
                           length(g.touch_pairs), pointer(a[4]), pointer(a[5]), pointer(a[6]), nw, pointer(a[7]),
                           wake === nothing ? 0 : length(wake.tris), pointer(a[8]),
                           wake === nothing ? 0 : length(wake.filaments), pointer(a[9])))
    end
    hs = fill(Ptr{Cvoid}(C_NULL), length(cases))
    sts = Vector{VpStats}(undef, length(cases))
    GC.@preserve keep check(ctx.h, ccall((:vp_assemble_batch, LIB), Cint,
        (Ptr{Cvoid}, Ref{VpOptions}, Cint, Ptr{VpInput}, Ptr{Ptr{Cvoid}}, Ptr{VpStats}),
        ctx.h, o, length(cases), ins, hs, sts))
    out = []
    for (k, (g, dm, σ, V∞, wake)) in enumerate(cases)
        nw = wake === nothing ? 0 : length(wake.x)
        A = DeviceSystem(ctx, hs[k], dm.nslot, dm.nslot + nw)
        finalizer(a -> ccall((:vp_system_free, LIB), Cvoid, (Ptr{Cvoid},), a.h), A)
        b = Vector{Cdouble}(undef, dm.nslot)
        check(ctx.h, ccall((:vp_system_download, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
            ctx.h, A.h, C_NULL, b))
        push!(out, (A, b, sts[k]))
    end
    return out
end

# the far tier's test triangles per tile (the autotuner's setting): 1, 2 or 4 in FP64, 2, 4 or 8 mixed
set_far_tile(ctx::Context, precision::Symbol, tile::Integer) = check(ctx.h, ccall((:vp_set_far_tile, LIB), Cint,
    (Ptr{Cvoid}, Cint, Cint), ctx.h, precision == :mixed ? 1 : 0, tile))
far_tile(ctx::Context, precision::Symbol) = ccall((:vp_get_far_tile, LIB), Cint, (Ptr{Cvoid}, Cint), ctx.h,
    precision == :mixed ? 1 : 0)

# ---- the bordered solve -----------------------------------------------------------------------------------------------

mutable struct GalerkinFactorization
    ctx::Context
    h::Ptr{Cvoid}
    dm::DOFMapping
    cond::Cdouble
end

function factorize_galerkin(dm::DOFMapping, A::DeviceSystem; W=nothing, precision::Symbol=:fp64)
    cp, cc, cv = csr(dm.C)
    wp, wc, wv = W === nothing ? (Cint[0], Cint[0], Cdouble[0]) : csr(W)
    h, cond = Ref{Ptr{Cvoid}}(C_NULL), Ref{Cdouble}()
    check(A.ctx.h, ccall((:vp_factorize, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cint},
         Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cdouble}, Ptr{Cint}, Ref{Ptr{Cvoid}}, Ref{Cdouble}),
        A.ctx.h, A.h, precision === :mixed ? 1 : 0, dm.nq, cp, cc, cv, W === nothing ? 0 : size(W, 1), wp, wc, wv,
        length(dm.body_closed), Cint.(q_body(dm)), collect(Cdouble, dm.slot_area), Cint.(dm.slot_body), h, cond))
    F = GalerkinFactorization(A.ctx, h[], dm, cond[])
    finalizer(f -> ccall((:vp_factor_free, LIB), Cvoid, (Ptr{Cvoid},), f.h), F)
end

"""solve_galerkin(F, b) (solve.jl:95-99); b may hold several right hand sides as columns"""
function solve_galerkin(F::GalerkinFactorization, b::AbstractVecOrMat)
    nrhs = size(b, 2)
    q = Matrix{Cdouble}(undef, F.dm.nq, nrhs)
    λ = Matrix{Cdouble}(undef, max(length(F.dm.body_closed), 1), nrhs)
    check(F.ctx.h, ccall((:vp_solve, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
        F.ctx.h, F.h, nrhs, Matrix{Cdouble}(reshape(b, :, nrhs)), q, λ))
    b isa AbstractVector && return (q=vec(q), μ=F.dm.C * vec(q), λ=vec(λ), cond=F.cond)
    return (q=q, μ=F.dm.C * q, λ=λ, cond=F.cond)
end

"""solve_galerkin(dm, A, b; W) (solve.jl:51-59), with the residual of the bordered system"""
function solve_galerkin(dm::DOFMapping, A::DeviceSystem, b::AbstractVector; W=nothing, precision::Symbol=:fp64)
    F = factorize_galerkin(dm, A; W, precision)
    q = Vector{Cdouble}(undef, dm.nq)
    λ = Vector{Cdouble}(undef, max(length(dm.body_closed), 1))
    res = Ref{Cdouble}()
    check(F.ctx.h, ccall((:vp_solve_system, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{Cdouble}), F.ctx.h, F.h, A.h, q, λ, res))
    return (q=q, μ=dm.C * q, λ=λ, cond=F.cond, residual=res[])
end

"""Mᵀ [ξ; η] = [g; 0] with the factors F (g: nq, or nq x k)"""
function solve_transposed(F::GalerkinFactorization, g::AbstractVecOrMat)
    k = size(g, 2)
    ξ = Matrix{Cdouble}(undef, F.dm.nq, k)
    check(F.ctx.h, ccall((:vp_solve_transposed, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}),
        F.ctx.h, F.h, k, Matrix{Cdouble}(reshape(g, :, k)), ξ))
    return g isa AbstractVector ? vec(ξ) : ξ
end

"""consistency(dm, A, b; W) (solve.jl:111-115) of the device's A and b"""
function consistency(dm::DOFMapping, A::DeviceSystem, b=nothing; W=nothing)
    cp, cc, cv = csr(dm.C)
    wp, wc, wv = W === nothing ? (Cint[0], Cint[0], Cdouble[0]) : csr(W)
    out = Vector{Cdouble}(undef, 3)
    check(A.ctx.h, ccall((:vp_consistency, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble},
         Ptr{Cdouble}),
        A.ctx.h, A.h, dm.nq, cp, cc, cv, W === nothing ? 0 : size(W, 1), wp, wc, wv, out))
    rhs = b === nothing ? out[3] : abs(sum(b)) / sum(abs, b)
    return (rows=out[1], columns=out[2], rhs=rhs)
end

# ---- loads (src/post/forces.jl, Post.jl), FP64 on the GPU ----------------------------------------------------------

corners(els) = collect(Cdouble, reduce(vcat, [vcat(el.x[1], el.x[2], el.x[3]) for el in els]))

"""u, Cp, F, M of the gradient route (Post.jl:72-84, forces.jl:11-20); dμdt (slots) for unsteady flow"""
function surface_loads(els, dm::DOFMapping, μ, V∞; dμdt=nothing, origin=zeros(3), ctx::Context=default_context())
    n = length(els)
    u, cp, F, M = Matrix{Cdouble}(undef, 3, n), Vector{Cdouble}(undef, n), zeros(3), zeros(3)
    check(ctx.h, ccall((:vp_surface_loads, LIB), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cint}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
         Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
        ctx.h, n, corners(els), idx0(dm.corner_slot), dm.nslot, collect(Cdouble, μ),
        dμdt === nothing ? C_NULL : collect(Cdouble, dμdt), collect(Cdouble, V∞), collect(Cdouble, origin), u, cp, F, M))
    return (u=[SVector{3}(c) for c in eachcol(u)], cp=cp, F=SVector{3}(F), M=SVector{3}(M))
end

"""pressure_force(els, cp; origin) (forces.jl:11-20)"""
function pressure_force(els, cp; origin=zeros(3), ctx::Context=default_context())
    F, M = zeros(3), zeros(3)
    check(ctx.h, ccall((:vp_pressure_force, LIB), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
        ctx.h, length(els), corners(els), collect(Cdouble, cp), collect(Cdouble, origin), F, M))
    return SVector{3}(F), SVector{3}(M)
end

function wake_loads(wte, μ_w, V∞; ctx::Context=default_context())
    ptr = Cint.(cumsum([0; length.(wte.lines)]))
    F, D = zeros(3), Ref{Cdouble}()
    check(ctx.h, ccall((:vp_wake_loads, LIB), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Ptr{Cdouble},
         Ptr{Cdouble}, Ref{Cdouble}),
        ctx.h, length(wte.x), flat(wte.x), length(wte.lines), ptr, Cint.(reduce(vcat, wte.lines) .- 1),
        Cint.(wte.closed), collect(Cdouble, μ_w), collect(Cdouble, V∞), F, D))
    return SVector{3}(F), D[]
end

kutta_joukowski_force(dm::DOFMapping, μ_w, V∞) = wake_loads(dm.wake_te, μ_w, V∞)[1]   # forces.jl:34-39
trefftz_drag(dm::DOFMapping, μ_w, V∞) = wake_loads(dm.wake_te, μ_w, V∞)[2]            # forces.jl:53-81

# ---- the adjoint as a ChainRulesCore.rrule -------------------------------------------------------------------------

"""
    wing_loads(g, dm, wake, W, α; S, opts, precision) -> (CL, CDi)

CL by the pressure route and CDi by the Trefftz plane of a wing with its rigid wake at angle of attack α (|V∞| = 1,
lift along (-sin α, 0, cos α), reference area S), through assemble, factorize_galerkin and solve_galerkin on the GPU.
Its rrule gives dCL/dx, dCDi/dx (all body nodes) and d/dα from the discrete adjoint: the transposed solve with the
same factors and the pair-integral derivatives of vp_adjoint.
"""
function wing_loads(g, dm, wake, W, α; S, opts=AssemblyOptions(), precision::Symbol=:mixed, ctx::Context=default_context())
    return first(wing_forward(g, dm, wake, W, α; S, opts, precision, ctx))
end

function wing_forward(g, dm, wake, W, α; S, opts, precision, ctx)
    V = SVector(cos(α), 0.0, sin(α))
    els = build_elements(g)
    σ = [-dot(el.n, V) for el in els]
    A, b, _ = assemble(g, dm, els, σ, V; opts, wake, precision, ctx)
    F = factorize_galerkin(dm, A; W, precision)
    sol = solve_galerkin(F, b)
    eL = SVector(-sin(α), 0.0, cos(α))
    loads = surface_loads(els, dm, sol.μ, V; ctx)
    μ_w = dm.K * sol.q
    CL = dot(loads.F, eL) / S
    CDi = trefftz_drag(dm, μ_w, V) / S
    return (CL=CL, CDi=CDi), (els=els, σ=σ, V=V, F=F, sol=sol, μ_w=μ_w)
end

"""
The explicit derivatives of the objectives at fixed doublets, by hand in reverse mode: CL = F·e_L/S with
F = -Σ Cp A n, Cp = 1 - |u|²/|V∞|², u = V∞ - (V∞·n)n + ∇μ (Post.jl:72-84, forces.jl:11-20), with respect to the slot
doublets μ, the body nodes and α; CDi = D/S with D the Trefftz drag (forces.jl:53-81) with respect to the trailing
edge doublets μ_w, the trailing edge nodes and α.
"""
function explicit_load_derivatives(g, dm, μ, μ_w, α, S)
    V, dV = SVector(cos(α), 0.0, sin(α)), SVector(-sin(α), 0.0, cos(α))
    eL, deL = dV, -V
    V2 = dot(V, V)
    dCL_dμ, dCL_dx, dCL_dα = zeros(dm.nslot), zeros(3, length(g.x)), 0.0
    for (t, tri) in enumerate(g.tris)
        a, b, c = g.x[tri[1]], g.x[tri[2]], g.x[tri[3]]
        cs = dm.corner_slot[t]
        m = SVector(μ[cs[1]], μ[cs[2]], μ[cs[3]])
        nA = cross(b - a, c - a)
        A2 = norm(nA)
        n = nA / A2
        e = (c - b, a - c, b - a)
        G = m[1] * e[1] + m[2] * e[2] + m[3] * e[3]
        i2 = 1 / A2^2
        gμ = cross(nA, G) * i2
        Vn = dot(n, V)
        u = V - Vn * n + gμ
        uu = dot(u, u)
        cp = 1 - uu / V2
        nAe = dot(nA, eL)
        # reverse
        cp_b = -nAe / (2S)
        nA_b = -(cp / (2S)) * eL
        u_b = (cp_b * (-2 / V2)) * u
        n_b = -Vn * u_b - dot(u_b, n) * V
        G_b = cross(u_b, nA) * i2
        trip = dot(u_b, gμ)
        nA_b += cross(G, u_b) * i2 - (2 * trip * i2) * nA
        for k in 1:3
            dCL_dμ[cs[k]] += dot(G_b, e[k])
        end
        xb = [zero(V), zero(V), zero(V)]
        for (k, (p, q)) in enumerate(((3, 2), (1, 3), (2, 1)))  # e_1 = c - b, e_2 = a - c, e_3 = b - a
            xb[p] += m[k] * G_b
            xb[q] -= m[k] * G_b
        end
        nA_b += (n_b - dot(n_b, n) * n) / A2
        u1, u2 = b - a, c - a
        u1_b, u2_b = cross(u2, nA_b), cross(nA_b, u1)
        xb[2] += u1_b
        xb[3] += u2_b
        xb[1] -= u1_b + u2_b
        for k in 1:3
            dCL_dx[:, tri[k]] .+= xb[k]
        end
        V_b = (u_b - dot(u_b, n) * n) + (cp_b * 2 * uu / V2^2) * V
        dCL_dα += dot(V_b, dV) + dot(-(cp / 2) * nA / S, deL)
    end
    # CDi: the Trefftz sum (O(nte²)) in reverse mode, over the strips and the trailing vortices
    wte = dm.wake_te
    d = V / norm(V)
    P(x) = x - dot(x, d) * d
    segs = [(l[i], l[mod1(i + 1, length(l))]) for (l, cl) in zip(wte.lines, wte.closed) for i in 1:(cl ? length(l) : length(l) - 1)]
    Γ = [(μ_w[a] + μ_w[b]) / 2 for (a, b) in segs]
    vort = Tuple{Int,Int,Int}[]  # (node, segment before or 0, segment after or 0)
    s0 = 0
    for (l, cl) in zip(wte.lines, wte.closed)
        m = length(l)
        ns = cl ? m : m - 1
        for i in 1:m
            push!(vort, (l[i], i > 1 ? s0 + i - 1 : (cl ? s0 + ns : 0), i <= ns ? s0 + i : 0))
        end
        s0 += ns
    end
    ΔΓ(v) = (v[3] > 0 ? Γ[v[3]] : 0.0) - (v[2] > 0 ? Γ[v[2]] : 0.0)
    k2 = 2 / V2 / S
    dCDi_dμw, dCDi_dxte = zeros(length(μ_w)), zeros(3, length(wte.x))
    Γ_b = zeros(length(Γ))
    CDi_x = zeros(3, length(wte.x))
    for (k, (a, b)) in enumerate(segs)
        pa, pb = P(wte.x[a]), P(wte.x[b])
        cc, ua = (pa + pb) / 2, pb - pa
        for v in vort
            r = cc - P(wte.x[v[1]])
            r2 = dot(r, r)
            h = dot(ua, r) / r2 / (4π)
            Γ_b[k] += k2 * h * ΔΓ(v)
            dG = k2 * Γ[k] * h
            v[3] > 0 && (Γ_b[v[3]] += dG)
            v[2] > 0 && (Γ_b[v[2]] -= dG)
            hb = k2 * Γ[k] * ΔΓ(v) / (4π)
            ua_b = (hb / r2) * r
            r_b = (hb / r2) * ua - (2 * hb * dot(ua, r) / r2^2) * r
            CDi_x[:, a] .+= -ua_b + r_b / 2
            CDi_x[:, b] .+= ua_b + r_b / 2
            CDi_x[:, v[1]] .-= r_b
        end
    end
    for (k, (a, b)) in enumerate(segs)
        dCDi_dμw[a] += Γ_b[k] / 2
        dCDi_dμw[b] += Γ_b[k] / 2
    end
    for j in axes(CDi_x, 2)  # the projection's derivative: P is linear, P' = I - d dᵀ
        pb = SVector{3}(CDi_x[:, j])
        dCDi_dxte[:, j] .= pb - dot(pb, d) * d
    end
    dCDi_dx = zeros(3, length(g.x))
    for (j, node) in enumerate(wte.node)
        dCDi_dx[:, node] .+= dCDi_dxte[:, j]
    end
    # α turns V∞ and so the projection direction d; D scales with 1/|V∞|² (|V∞| = 1 here)
    dd = (dV - dot(dV, d) * d) / norm(V)
    d_b = zeros(3)
    for j in axes(CDi_x, 2)
        x = wte.x[j]
        pb = SVector{3}(CDi_x[:, j])
        d_b .-= dot(pb, d) * x + dot(x, d) * pb
    end
    dCDi_dα = dot(d_b, dd)
    return (dCL_dμ=dCL_dμ, dCL_dx=dCL_dx, dCL_dα=dCL_dα, dCDi_dμw=dCDi_dμw, dCDi_dx=dCDi_dx, dCDi_dα=dCDi_dα)
end

"""d/dx, d/dwx, d/dα of νᵀ(A(x) μ - b(x)) for one or two adjoint vectors ν (nslot x k), vp_adjoint"""
function pair_derivatives(g, dm, wake, σ, V, dV, ν::AbstractMatrix, μ::AbstractVector; opts=AssemblyOptions(),
    precision::Symbol=:mixed, ctx::Context=default_context())
    k = size(ν, 2)
    nw = wake === nothing ? 0 : length(wake.x)
    gx, gw, dα = zeros(3, length(g.x), k), zeros(3, max(nw, 1), k), zeros(k)
    tp = isempty(g.touch_pairs) ? Cint[0, 0] : idx0(g.touch_pairs)
    wx = wake === nothing ? Cdouble[0] : flat(wake.x)
    wt = wake === nothing || isempty(wake.tris) ? Cint[0, 0, 0] : idx0(wake.tris)
    wf = wake === nothing || isempty(wake.filaments) ? Cint[0, 0] : idx0(wake.filaments)
    check(ctx.h, ccall((:vp_adjoint, LIB), Cint,
        (Ptr{Cvoid}, Ref{VpOptions}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Ptr{Cint}, Cint, Cint, Ptr{Cint},
         Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cdouble},
         Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{VpStats}),
        ctx.h, Ref(VpOptions(opts; precision)), length(g.x), flat(g.x), length(g.tris), idx0(g.tris),
        idx0(dm.corner_slot), dm.nslot, length(g.touch_pairs), tp, collect(Cdouble, σ), collect(Cdouble, V), nw, wx,
        wake === nothing ? 0 : length(wake.tris), wt, wake === nothing ? 0 : length(wake.filaments), wf, k,
        Matrix{Cdouble}(ν), collect(Cdouble, μ), collect(Cdouble, dV), gx, gw, dα, C_NULL))
    return gx, gw[:, 1:nw, :], dα
end

"""the wake nodes move with their trailing edge nodes: their derivatives go to those body nodes"""
function wake_to_te(dm, wake, gw)
    out = zeros(3, size(gw, 2) == 0 ? 0 : maximum(dm.wake_te.node))
    for (j, te) in enumerate(wake.te)
        out[:, dm.wake_te.node[te]] .+= gw[:, j]
    end
    return out
end

function ChainRulesCore.rrule(::typeof(wing_loads), g, dm, wake, W, α; S, opts=AssemblyOptions(), precision::Symbol=:mixed,
    ctx::Context=default_context())
    y, st = wing_forward(g, dm, wake, W, α; S, opts, precision, ctx)
    # the explicit derivatives of CL (pressure route) and CDi (Trefftz) at fixed doublets
    ∂ = explicit_load_derivatives(g, dm, st.sol.μ, st.μ_w, α, S)
    function pullback(Δ)
        ΔCL, ΔCDi = Δ.CL, Δ.CDi
        gq = ΔCL * (transpose(dm.C) * ∂.dCL_dμ) + ΔCDi * (transpose(dm.K) * ∂.dCDi_dμw)
        ξ = solve_transposed(st.F, gq)
        μcols = W === nothing ? st.sol.μ : vcat(st.sol.μ, W * st.sol.q)
        dV = SVector(-sin(α), 0.0, cos(α))
        gx, gw, dα = pair_derivatives(g, dm, wake, st.σ, st.V, dV, reshape(dm.C * ξ, :, 1), μcols; opts, precision, ctx)
        dx = ΔCL * ∂.dCL_dx + ΔCDi * ∂.dCDi_dx - gx[:, :, 1]
        wake === nothing || (dx[:, 1:size(wake_to_te(dm, wake, gw[:, :, 1]), 2)] .-= wake_to_te(dm, wake, gw[:, :, 1]))
        return NoTangent(), dx, NoTangent(), NoTangent(), NoTangent(), ΔCL * ∂.dCL_dα + ΔCDi * ∂.dCDi_dα - dα[1]
    end
    return y, pullback
end

# ---- the free wake on the GPU ---------------------------------------------------------------------------------------

# vp_freewake_setup (vortexpanel_gpu.h): the resolved options, the body and its factors, the DOF map, the topology and
# the trailing edge panel; pointers stay valid for the call (GC.@preserve)
struct VpFreeWakeSetup
    dt::Cdouble
    keep_rows::Cint
    core_mode::Cint
    overlap::Cdouble
    core_factor::Cdouble
    core_floor::Cdouble
    core_value::Cdouble
    advection::Cint
    delete_limit::Cdouble
    assembly::VpOptions
    nnode::Cint
    x::Ptr{Cdouble}
    ntri::Cint
    tris::Ptr{Cint}
    corner_slot::Ptr{Cint}
    nslot::Cint
    sigma::Ptr{Cdouble}
    vinf::Ptr{Cdouble}
    factor::Ptr{Cvoid}
    b0::Ptr{Cdouble}
    nq::Cint
    C_rowptr::Ptr{Cint}
    C_col::Ptr{Cint}
    C_val::Ptr{Cdouble}
    nte::Cint
    K_rowptr::Ptr{Cint}
    K_col::Ptr{Cint}
    K_val::Ptr{Cdouble}
    te_x::Ptr{Cdouble}
    nline::Cint
    line_ptr::Ptr{Cint}
    line_nodes::Ptr{Cint}
    line_closed::Ptr{Cint}
    nstrip::Cint
    strips::Ptr{Cint}
    nfirst::Cint
    first_nodes::Ptr{Cint}
    nlast::Cint
    last_nodes::Ptr{Cint}
    edge::Ptr{Cdouble}
    npw::Cint
    pw_x::Ptr{Cdouble}
    pw_te::Ptr{Cint}
    npt::Cint
    pt_tris::Ptr{Cint}
    npf::Cint
    pf::Ptr{Cint}
    merge::Ptr{Cint}
    particle_capacity::Cint
end

struct VpFreeWakeRecord
    n::Cint
    t::Cdouble
    F_pressure::NTuple{3,Cdouble}
    M_pressure::NTuple{3,Cdouble}
    F_kj::NTuple{3,Cdouble}
    F_impulse::NTuple{3,Cdouble}
    Ω::NTuple{3,Cdouble}
    I::NTuple{3,Cdouble}
    rows::Cint
    particles::Cint
    λ::Cdouble
    umax::Cdouble
end

struct VpFreeWakeCounts
    n::Cint
    t::Cdouble
    nrows::Cint
    nparticles::Cint
    conversions::Cint
    I_prev::NTuple{3,Cdouble}
end

"""FreeWakeSim (step.jl:35-58) with its state on the GPU; step! and run! as the reference's"""
mutable struct GPUFreeWakeSim
    ctx::Context
    h::Ptr{Cvoid}
    F::GalerkinFactorization
    nte::Int
    history::Vector{Any}
end

function GPUFreeWakeSim(g::SurfaceGeometry, dm::DOFMapping, V∞::SVector{3}; opts::FreeWakeOptions,
    assembly::AssemblyOptions=AssemblyOptions(), precision::Symbol=:fp64, capacity::Integer=4096,
    ctx::Context=default_context())
    els = build_elements(g)
    σ = [-dot(el.n, V∞) for el in els]
    te = te_panel(g, dm, V∞; length=something(opts.te_len, 0.3 * norm(V∞) * opts.dt), direction=opts.te_direction)
    A, b0, _ = assemble(g, dm, els, σ, V∞; opts=assembly, wake=te, precision, ctx)
    F = factorize_galerkin(dm, A; W=wake_rows(dm, te.te), precision)
    topo = FreeWake.Topology(dm)
    edge = [te.x[topo.nte+k] for k in 1:topo.nte]
    core = FreeWake.CoreRule(opts, V∞)
    row = norm(V∞) * opts.dt
    keep = opts.max_rows === :auto ? max(0, ceil(Int, (3 * FreeWake.first_core(core, edge, topo, row) - te.rows[2]) / row - 0.5)) :
           opts.max_rows
    widths = [norm(edge[B] - edge[A]) for (A, B) in topo.segments]
    merge = opts.merge_rows === :auto ? Cint[max(1, round(Int, w / row)) for w in widths] :
            opts.merge_rows == 1 ? nothing : fill(Cint(opts.merge_rows), length(widths))
    d = normalize(V∞)
    limit = isfinite(opts.delete_beyond) ? maximum(dot(x, d) for x in edge) + opts.delete_beyond * te.span : Inf
    mode = opts.core === :auto ? 0 : opts.core === :scaled ? 1 : 2
    C, K = csr(dm.C), csr(dm.K)
    x, tris, cs = flat(g.x), idx0(g.tris), idx0(dm.corner_slot)
    σv, Vv = collect(Cdouble, σ), collect(Cdouble, V∞)
    tex = flat(dm.wake_te.x)
    lp, ln, lc = Cint.(cumsum([0; length.(dm.wake_te.lines)])), Cint.(reduce(vcat, dm.wake_te.lines) .- 1), Cint.(dm.wake_te.closed)
    st = Cint.(reduce(vcat, [[a, b] for (a, b) in topo.segments]) .- 1)
    fn, lnodes = Cint.(topo.first_nodes .- 1), Cint.(topo.last_nodes .- 1)
    ed, pwx, pwte = flat(edge), flat(te.x), Cint.(te.te .- 1)
    ptt = isempty(te.tris) ? Cint[0, 0, 0] : idx0(te.tris)
    pff = isempty(te.filaments) ? Cint[0, 0] : idx0(te.filaments)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve x tris cs σv Vv b0 C K tex lp ln lc st fn lnodes ed pwx pwte ptt pff merge begin
        s = VpFreeWakeSetup(opts.dt, keep, mode, opts.overlap, opts.core_factor, core.floor, mode == 2 ? opts.core : 0.0,
            opts.advection === :free ? 0 : 1, limit, VpOptions(assembly; precision), length(g.x), pointer(x),
            length(g.tris), pointer(tris), pointer(cs), dm.nslot, pointer(σv), pointer(Vv), F.h, pointer(b0), dm.nq,
            pointer(C[1]), pointer(C[2]), pointer(C[3]), topo.nte, pointer(K[1]), pointer(K[2]), pointer(K[3]),
            pointer(tex), length(dm.wake_te.lines), pointer(lp), pointer(ln), pointer(lc), length(topo.segments),
            pointer(st), length(fn), pointer(fn), length(lnodes), pointer(lnodes), pointer(ed), length(te.x),
            pointer(pwx), pointer(pwte), length(te.tris), pointer(ptt), length(te.filaments), pointer(pff),
            merge === nothing ? Ptr{Cint}(C_NULL) : pointer(merge), capacity)
        check(ctx.h, ccall((:vp_freewake_create, LIB), Cint, (Ptr{Cvoid}, Ref{VpFreeWakeSetup}, Ref{Ptr{Cvoid}}),
            ctx.h, s, h))
    end
    sim = GPUFreeWakeSim(ctx, h[], F, topo.nte, Any[])
    finalizer(s -> ccall((:vp_freewake_free, LIB), Cvoid, (Ptr{Cvoid},), s.h), sim)
end

"""step!(sim) (step.jl:113-146) on the GPU: the step's record"""
function step!(sim::GPUFreeWakeSim)
    r = Ref{VpFreeWakeRecord}()
    check(sim.ctx.h, ccall((:vp_freewake_step, LIB), Cint, (Ptr{Cvoid}, Ref{VpFreeWakeRecord}), sim.h, r))
    μ_w = Vector{Cdouble}(undef, sim.nte)
    check(sim.ctx.h, ccall((:vp_freewake_get_state, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cint}, Ptr{Int8}, Ptr{Cint},
         Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
        sim.h, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, μ_w, C_NULL))
    x = r[]
    rec = (n=x.n, t=x.t, μ_w=μ_w, F_pressure=SVector(x.F_pressure), M_pressure=SVector(x.M_pressure),
        F_kj=SVector(x.F_kj), F_impulse=SVector(x.F_impulse), Ω=SVector(x.Ω), I=SVector(x.I), rows=x.rows,
        particles=x.particles, λ=x.λ, umax=x.umax)
    push!(sim.history, rec)
    return rec
end

"""run!(sim, n) (step.jl:205-216)"""
function run!(sim::GPUFreeWakeSim, nsteps::Integer; progress=nothing)
    for _ in 1:nsteps
        rec = step!(sim)
        progress === nothing || progress(sim, rec)
    end
    return sim.history
end

"""the counts of the simulation (steps, time, node rows, particles, conversions)"""
function counts(sim::GPUFreeWakeSim)
    c = Ref{VpFreeWakeCounts}()
    check(sim.ctx.h, ccall((:vp_freewake_info, LIB), Cint, (Ptr{Cvoid}, Ref{VpFreeWakeCounts}), sim.h, c))
    return c[]
end

end # module
