"""
    SMGPU

Julia binding of libsmgpu.so for NuclearToolkit.jl's ShellModel path.

`SMGPU.main_sm(sntf, target_nuc, num_ev, target_J; q=1, is_block=false,
lm=300, ls=20, tol=1e-8, precision=:fp64)` has the arguments and the return
value of `NuclearToolkit.main_sm` (src/ShellModel/shellmodel_main.jl:89-281):
it returns the lowest `num_ev` eigenvalues and prints the J labels as the
reference does; `target_J = [2J]` runs the J-projected double Lanczos and
`is_block = true` the block Lanczos with block size `q`.  Parsing, basis,
jump tables, H·v and the Lanczos iterations run inside the library (GPU);
Julia passes the file name and receives the energies.

Set `ENV["SMGPU_LIB"]` to the path of libsmgpu.so before loading the module.
"""
module SMGPU

const libsmgpu = get(ENV, "SMGPU_LIB", "libsmgpu.so")

const SMGPU_OK = Cint(0)
const SMGPU_ERR_NOCONV = Cint(-8)
const PRECISION = Dict(:fp64 => Cint(0), :mixed => Cint(1))

last_error(h::Ptr{Cvoid}) = unsafe_string(ccall((:smgpu_last_error, libsmgpu), Cstring, (Ptr{Cvoid},), h))

function check(rc::Cint, h::Ptr{Cvoid})
    rc == SMGPU_OK && return nothing
    error("libsmgpu error $(rc): $(last_error(h))")
end

"""Create a problem handle (readsmsnt + basis + jump tables on the GPU);
`twoJ >= 0` builds the basis of Mtot = twoJ (main_sm's target_J = [twoJ])."""
function create(sntf::AbstractString, target_nuc::AbstractString; precision::Symbol=:fp64, twoJ::Int=-1)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    if twoJ < 0
        rc = ccall((:smgpu_problem_create_from_snt, libsmgpu), Cint,
                   (Cstring, Cstring, Cint, Ref{Ptr{Cvoid}}), sntf, target_nuc, PRECISION[precision], ref)
    else
        rc = ccall((:smgpu_problem_create_from_snt_J, libsmgpu), Cint,
                   (Cstring, Cstring, Cint, Cint, Ref{Ptr{Cvoid}}), sntf, target_nuc, twoJ, PRECISION[precision], ref)
    end
    check(rc, C_NULL)
    return ref[]
end

destroy(h::Ptr{Cvoid}) = ccall((:smgpu_problem_destroy, libsmgpu), Cint, (Ptr{Cvoid},), h)

function mdim(h::Ptr{Cvoid})
    md = Ref{Clonglong}(0); nb = Ref{Cint}(0)
    check(ccall((:smgpu_dims, libsmgpu), Cint, (Ptr{Cvoid}, Ref{Clonglong}, Ref{Cint}, Ptr{Clonglong}),
                h, md, nb, C_NULL), h)
    return Int(md[])
end

"""twf .+= H * wf, the semantics of operate_H! (lanczos_methods.jl:153)."""
function operate_H!(h::Ptr{Cvoid}, wf::Vector{Float64}, twf::Vector{Float64})
    check(ccall((:smgpu_matvec, libsmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Cint, Cint),
                h, wf, twf, 1, 1), h)
    return nothing
end

"""<v|J^2|v> for the columns of a Vector of vectors (operate_J! + dot)."""
function jj(h::Ptr{Cvoid}, vecs::Vector{Vector{Float64}})
    m = mdim(h)
    flat = Vector{Float64}(undef, m * length(vecs))
    for (k, v) in enumerate(vecs); flat[(k-1)*m+1:k*m] .= v; end
    out = zeros(Float64, length(vecs))
    check(ccall((:smgpu_jj, libsmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{Float64}),
                h, flat, length(vecs), out), h)
    return out
end

"""<vl_a| O |vr_b> of the one-body M1 (op = 0) or E2 (op = 1) operator
(smgpu_obtr): symmetric = true is eval_moment's form on one basis
(transit.jl:82-284), false transit_main's from hr's basis to hl's
(transit.jl:286-531).  Returns an nl x nr matrix."""
function obtr(hl::Ptr{Cvoid}, hr::Ptr{Cvoid}, op::Integer, vl::Vector{Vector{Float64}},
              vr::Vector{Vector{Float64}}; symmetric::Bool=true,
              gfactors=[1.0, 0.0, 5.586, -3.826], effcharge=[1.5, 0.5])
    fl = reduce(vcat, vl); fr = reduce(vcat, vr)
    out = zeros(Float64, length(vr), length(vl))   # C row-major nl x nr
    check(ccall((:smgpu_obtr, libsmgpu), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint,
                 Ptr{Float64}, Cint, Ptr{Float64}),
                hl, hr, op, symmetric ? 1 : 0, Vector{Float64}(gfactors), Vector{Float64}(effcharge),
                fl, length(vl), fr, length(vr), out), hl)
    return permutedims(out)
end

"""Nmat and the transition densities of prepEC mode "TD" (smgpu_ec_td,
eigenvector_continuation.jl:212-310): TDs[:, Nij] = [OBTD_p; OBTD_n; TBTD]."""
function ec_td(h::Ptr{Cvoid}, vecs::Vector{Vector{Float64}})
    n = length(vecs)
    ltd = Ref{Cint}(0)
    check(ccall((:smgpu_ec_td_length, libsmgpu), Cint, (Ptr{Cvoid}, Ref{Cint}), h, ltd), h)
    nmat = zeros(Float64, n, n)
    tds = zeros(Float64, Int(ltd[]), div(n * (n + 1), 2))
    check(ccall((:smgpu_ec_td, libsmgpu), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{Float64}, Ptr{Float64}),
                h, reduce(vcat, vecs), n, nmat, tds), h)
    return nmat, tds
end

# shellmodel_main.jl:1105-1113
function J_from_JJ1(JJ, tol=1.e-6)
    for J = 0:100
        hJ = 0.5 * J
        abs(hJ * (hJ + 1.0) - JJ) < tol && return hJ
    end
    return -1.0
end

function main_sm(sntf, target_nuc, num_ev, target_J; q=1, is_block=false, lm=300, ls=20, tol=1.e-8,
                 max_restarts=10000, precision::Symbol=:fp64, is_show=false)
    length(target_J) <= 1 || error("Invalid `target_J` Multiple J is not supported now.")
    tJ = length(target_J) == 1 ? Int(target_J[1]) : -1
    (is_block && tJ >= 0) && error("SMGPU: block Lanczos with target_J is not in the GPU library")
    h = create(sntf, target_nuc; precision=precision, twoJ=tJ)
    try
        m = mdim(h)
        n = min(num_ev, m)
        en = zeros(Float64, n)
        vecs = zeros(Float64, n * m)
        stats = zeros(Cint, 8)
        argt = (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Cint})
        if is_block
            rc = ccall((:smgpu_solve_block, libsmgpu), Cint, argt,
                       h, q, num_ev, lm, ls, tol, max_restarts, C_NULL, en, vecs, stats)
        elseif tJ >= 0
            rc = ccall((:smgpu_solve_J, libsmgpu), Cint, argt,
                       h, tJ, num_ev, lm, ls, tol, max_restarts, C_NULL, en, vecs, stats)
        else
            rc = ccall((:smgpu_solve, libsmgpu), Cint,
                       (Ptr{Cvoid}, Cint, Cint, Cint, Cdouble, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Cint}),
                       h, num_ev, lm, ls, tol, max_restarts, C_NULL, en, vecs, stats)
        end
        rc == SMGPU_ERR_NOCONV && @warn "Lanczos not converged after $(max_restarts) restarts"
        rc == SMGPU_ERR_NOCONV || check(rc, h)
        totJs = J_from_JJ1.(jj(h, [vecs[(k-1)*m+1:k*m] for k = 1:n]))
        if tJ < 0
            println("J $totJs")
            print("En. "); foreach(x -> print(lpad(string(round(x, digits=4)), 10), " "), en); print("\n")
        else
            print("2J= $(Int(2*totJs[1]))  En."); foreach(x -> print(lpad(string(round(x, digits=5)), 12), " "), en)
            print("\n")
        end
        is_show && println("matvecs $(stats[2]) restarts $(stats[3])")
        return en
    finally
        destroy(h)
    end
end

end # module
