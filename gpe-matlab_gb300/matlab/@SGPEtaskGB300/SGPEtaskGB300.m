classdef SGPEtaskGB300 < GPEtaskGB300
    %SGPEtaskGB300 - SGPEtask (stochastic GPE) whose solve_split runs on a
    %GB300 GPU through libgpe (gpe_mex 'sgpe' -> gpe_solve_sgpe).
    %
    % Properties as SGPEtask (T, ecut, snapshots, ss_maxlength) plus seed, the
    % key of the counter-based noise stream (MATLAB's global randn stream is
    % not used, so a run is reproducible from its seed).  groundstate_itp and
    % get_energy are the GPEtaskGB300 ones.  Scalar omega must be 0: the
    % rotating SGPE (its Lz Crank-Nicolson branch) is not supported.
    %
    % UNVERIFIED: no MATLAB was available where this file was written; the
    % library call it makes is covered by the Python tests of the same ABI.

    properties
        T = 0               % temperature
        snapshots = {}      % kept for SGPEtask compatibility
        ss_maxlength = 100
        ecut = 0            % cut-off energy (applies when T > 0)
        seed = 0            % noise stream key (64-bit integer value)
    end

    methods
        function obj = SGPEtaskGB300(grid, trappot)
            obj@GPEtaskGB300(grid, trappot);
        end

        function phi = solve_split(task, ddt, niter_inner, niter_outer)
            % @SGPEtask/solve_split.m semantics, executed by libgpe.
            task.dispstat('', 'init');
            tic;
            task.gb300_push();
            if task.current_iter > 0
                phi = task.current_state;
            else
                phi = task.init_state;
            end
            gpe_mex('set_state', task.gb300_handle, complex(gather(phi)));
            timedep = isa(task.Vtd, 'function_handle') || numel(task.V0) > 1;
            if ~timedep
                gpe_mex('set_potential', task.gb300_handle, double(gather(task.Vtrap)));
            end
            gpe_mex('sgpe', task.gb300_handle, ddt, niter_inner, niter_outer, task, timedep, ...
                double(task.T), double(task.ecut), double(task.seed));
            phi = task.current_state;
        end
    end
end
